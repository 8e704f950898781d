#include "sDbscan.h"

#include <cmath>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

int dist_code(const std::string& s) {
    if (s == "Cosine") return SDB_COSINE;
    if (s == "L1") return SDB_L1;
    if (s == "L2") return SDB_L2;
    if (s == "Chi2") return SDB_CHI2;
    if (s == "JS") return SDB_JS;
    throw std::invalid_argument("Error: The distance is not support: " + s);
}

const char* dist_str(int c) {
    static const char* names[] = {"Cosine", "L1", "L2", "Chi2", "JS"};
    return (c >= 0 && c <= 4) ? names[c] : "?";
}

std::string int2str(long x) { return std::to_string(x); }

}  // namespace

sDbscan::sDbscan(int n, int d, int device) : n_(n), d_(d) {
    sdb_params_default(&prm_);
    prm_.topK = 5;        // C++ default of set_params (src/sDbscan.h:79)
    prm_.n_threads = 8;
    check(sdb_engine_create(n, d, device, &eng_), "sDbscan(n, d)");
}

sDbscan::~sDbscan() {
    if (eng_) sdb_engine_destroy(eng_);
}

void sDbscan::check(sdb_status s, const char* what) {
    if (s == SDB_OK) return;
    std::string msg = std::string(what) + " failed";
    if (eng_) {
        const char* e = sdb_last_error(eng_);
        if (e && *e) msg += std::string(": ") + e;
    } else {
        msg += " (status " + std::to_string((int)s) + ")";
    }
    if (s == SDB_ERR_ARG || s == SDB_ERR_NEGATIVE || s == SDB_ERR_ZERO_POINT) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

void sDbscan::push_params() { check(sdb_set_params(eng_, &prm_), "set_params"); }

void sDbscan::set_params(int numProj, int k, int m, std::string dist, int kerDim, float kerSigma, float kerSam,
                         int noiseClustering, float prob, bool ver, std::string filename, int numThreads,
                         int randomSeed) {
    prm_.n_proj = numProj;
    prm_.topK = k;
    prm_.topM = m;
    prm_.distance = dist_code(dist);
    prm_.ker_n_features = kerDim;
    prm_.ker_sigma = kerSigma;
    prm_.ker_intervalSampling = kerSam;
    prm_.clusterNoise = noiseClustering;
    prm_.samplingProb = prob;
    prm_.verbose = ver ? 1 : 0;
    prm_.n_threads = numThreads;
    prm_.random_seed = randomSeed;
    output_ = filename;
    push_params();
}

void sDbscan::set_kernel_params(std::string dist, int kerDim, float kerSigma, float kerSam) {
    prm_.distance = dist_code(dist);
    prm_.ker_n_features = kerDim;
    prm_.ker_sigma = kerSigma;
    prm_.ker_intervalSampling = kerSam;
    push_params();
}

void sDbscan::clear() {
    labels_.clear();
    n_clusters_ = 0;
    ordering_.clear();
    reachability_.clear();
    sdb_clear(eng_);
}

void sDbscan::set_topM(int m) { prm_.topM = m; push_params(); }
void sDbscan::set_topK(int k) { prm_.topK = k; push_params(); }
void sDbscan::set_proj(int p) { prm_.n_proj = p; push_params(); }
void sDbscan::set_clusterNoise(int c) { prm_.clusterNoise = c; push_params(); }
void sDbscan::set_threads(int t) { prm_.n_threads = t; }
void sDbscan::set_precision(int precision) {
    check(sdb_set_precision(eng_, precision), "set_precision");
    prm_.precision = precision;
}

void sDbscan::fit_sDbscan(const float* X, float eps, int minPts) {
    check(sdb_fit_sdbscan(eng_, X, eps, minPts), "fit_sDbscan");
    labels_.assign(n_, -1);
    int32_t nc = 0;
    check(sdb_get_labels(eng_, labels_.data(), &nc), "fit_sDbscan (labels)");
    n_clusters_ = nc;
    if (prm_.verbose) {  // output file written when verbose (src/sDbscan.cpp:878-889)
        const std::string f = output_ + "_" + dist_str(prm_.distance) + "_Eps_" + int2str(std::lround(1000 * eps)) +
                              "_MinPts_" + int2str(minPts) + "_KerFeatures_" +
                              int2str(prm_.distance == SDB_COSINE ? d_ : prm_.ker_n_features) + "_NumProj_" +
                              int2str(prm_.n_proj) + "_TopM_" + int2str(prm_.topM) + "_TopK_" + int2str(prm_.topK);
        std::ofstream out(f);
        for (int v : labels_) out << v << '\n';
    }
}

// loadtxtData (src/Utilities.cpp:57-95) through the engine library's loader.
static std::vector<float> load_txt(const std::string& dataset, int n, int d) {
    std::vector<float> X((size_t)n * d);
    if (sdb_load_txt(dataset.c_str(), n, d, X.data()) != SDB_OK)
        throw std::runtime_error("Error: Data file does not exist or holds fewer than n_points x n_features numbers: " +
                                 dataset);
    return X;
}

void sDbscan::load_fit_sDbscan(const std::string& dataset, float eps, int minPts) {
    const std::vector<float> X = load_txt(dataset, n_, d_);
    fit_sDbscan(X.data(), eps, minPts);
}

void sDbscan::load_fit_sOptics(const std::string& dataset, float eps, int minPts) {
    const std::vector<float> X = load_txt(dataset, n_, d_);
    fit_sOptics(X.data(), eps, minPts);
}

void sDbscan::test_sDbscan(const float* X, float eps, float rangeEps, int n_tests, int minPts) {
    if (n_tests < 1) throw std::runtime_error("test_sDbscan: n_tests must be >= 1");
    std::vector<float> E(n_tests);
    for (int i = 0; i < n_tests; ++i) E[i] = (float)(eps + 1.0 * i * rangeEps);  // src/sDbscan.cpp:1012
    std::vector<int32_t> L((size_t)n_tests * n_);
    std::vector<int32_t> ncl(n_tests);
    check(sdb_fit_sdbscan_sweep(eng_, X, E.data(), n_tests, minPts, L.data(), ncl.data()), "test_sDbscan");
    for (int i = 0; i < n_tests; ++i) {  // one labels file per eps (src/sDbscan.cpp:1026-1036)
        const std::string f = output_ + "_" + dist_str(prm_.distance) + "_Eps_" + int2str(std::lround(1000 * E[i])) +
                              "_MinPts_" + int2str(minPts) + "_KerFeatures_" +
                              int2str(prm_.distance == SDB_COSINE ? d_ : prm_.ker_n_features) + "_NumProj_" +
                              int2str(prm_.n_proj) + "_TopM_" + int2str(prm_.topM) + "_TopK_" + int2str(prm_.topK);
        std::ofstream out(f);
        for (int j = 0; j < n_; ++j) out << L[(size_t)i * n_ + j] << '\n';
    }
    labels_.assign(L.end() - n_, L.end());
    n_clusters_ = ncl.back();
}

void sDbscan::load_test_sDbscan(const std::string& dataset, float eps, float rangeEps, int n_tests, int minPts) {
    const std::vector<float> X = load_txt(dataset, n_, d_);
    test_sDbscan(X.data(), eps, rangeEps, n_tests, minPts);
}

void sDbscan::fit_sOptics(const float* X, float eps, int minPts) {
    check(sdb_fit_soptics(eng_, X, eps, minPts), "fit_sOptics");
    ordering_.assign(n_, 0);
    reachability_.assign(n_, 0.0f);
    check(sdb_get_optics(eng_, ordering_.data(), reachability_.data()), "fit_sOptics (results)");
    if (!output_.empty()) {  // src/sDbscan.cpp:1757-1768, format of src/Utilities.cpp:34-47
        const std::string f = output_ + "_" + dist_str(prm_.distance) + "_Eps_" + int2str(std::lround(1000 * eps)) +
                              "_MinPts_" + int2str(minPts) + "_NumEmbed_" +
                              int2str(prm_.distance == SDB_COSINE ? d_ : prm_.ker_n_features) + "_NumProj_" +
                              int2str(prm_.n_proj) + "_TopM_" + int2str(prm_.topM) + "_TopK_" + int2str(prm_.topK);
        std::ofstream out(f);
        for (size_t i = 0; i < ordering_.size(); ++i) out << ordering_[i] << " " << reachability_[i] << '\n';
    }
}

// ---- sngDbscan / sngOptics ------------------------------------------------------

void sDbscan::set_sngParams(std::string dist, float prob, int noiseClustering, bool ver, std::string filename,
                            int numThreads, int randomSeed) {
    const int code = dist_code(dist);
    check(sdb_set_sng_params(eng_, code, prob, noiseClustering, ver ? 1 : 0, numThreads, randomSeed), "set_sngParams");
    prm_.distance = code;
    prm_.samplingProb = prob;
    if (noiseClustering > 0) prm_.clusterNoise = 2;  // src/sDbscan.h:133-134
    prm_.verbose = ver ? 1 : 0;
    prm_.n_threads = numThreads;
    prm_.random_seed = randomSeed;
    output_ = filename;
}

// Output name of the sng fits (src/sDbscan.cpp:1171-1175, :1232-1236, :1872-1876).
std::string sDbscan::sng_file(float eps, int minPts) const {
    return output_ + "_" + dist_str(prm_.distance) + "_Eps_" + int2str(std::lround(1000 * eps)) + "_MinPts_" +
           int2str(minPts) + "_Prob_" + int2str(std::lround(1000 * prm_.samplingProb));
}

void sDbscan::fit_sngDbscan(const float* X, float eps, int minPts) {
    check(sdb_fit_sngdbscan(eng_, X, eps, minPts), "fit_sngDbscan");
    prm_.clusterNoise = 0;  // src/sDbscan.cpp:1157
    labels_.assign(n_, -1);
    int32_t nc = 0;
    check(sdb_get_labels(eng_, labels_.data(), &nc), "fit_sngDbscan (labels)");
    n_clusters_ = nc;
    if (prm_.verbose) {  // src/sDbscan.cpp:1170-1178
        std::ofstream out(sng_file(eps, minPts));
        for (int v : labels_) out << v << '\n';
    }
}

void sDbscan::test_sngDbscan(const float* X, float eps, float rangeEps, int n_tests, int minPts) {
    if (n_tests < 1) throw std::runtime_error("test_sngDbscan: n_tests must be >= 1");
    std::vector<float> E(n_tests);
    for (int i = 0; i < n_tests; ++i) E[i] = (float)(eps + 1.0 * i * rangeEps);  // src/sDbscan.cpp:1221
    std::vector<int32_t> L((size_t)n_tests * n_);
    std::vector<int32_t> ncl(n_tests);
    check(sdb_fit_sngdbscan_sweep(eng_, X, E.data(), n_tests, minPts, L.data(), ncl.data()), "test_sngDbscan");
    for (int i = 0; i < n_tests; ++i) {  // one labels file per eps (src/sDbscan.cpp:1232-1238)
        std::ofstream out(sng_file(E[i], minPts));
        for (int j = 0; j < n_; ++j) out << L[(size_t)i * n_ + j] << '\n';
    }
    labels_.assign(L.end() - n_, L.end());
    n_clusters_ = ncl.back();
}

void sDbscan::load_test_sngDbscan(const std::string& dataset, float eps, float rangeEps, int n_tests, int minPts) {
    const std::vector<float> X = load_txt(dataset, n_, d_);
    test_sngDbscan(X.data(), eps, rangeEps, n_tests, minPts);
}

void sDbscan::fit_sngOptics(const float* X, float eps, int minPts) {
    check(sdb_fit_sngoptics(eng_, X, eps, minPts), "fit_sngOptics");
    ordering_.assign(n_, 0);
    reachability_.assign(n_, 0.0f);
    check(sdb_get_optics(eng_, ordering_.data(), reachability_.data()), "fit_sngOptics (results)");
    if (!output_.empty()) {  // src/sDbscan.cpp:1871-1879
        std::ofstream out(sng_file(eps, minPts));
        for (size_t i = 0; i < ordering_.size(); ++i) out << ordering_[i] << " " << reachability_[i] << '\n';
    }
}

void sDbscan::load_fit_sngOptics(const std::string& dataset, float eps, int minPts) {
    const std::vector<float> X = load_txt(dataset, n_, d_);
    fit_sngOptics(X.data(), eps, minPts);
}
