// C-ABI probe around the UNMODIFIED reference class `sDbscan`
// (src/sDbscan.h:10-223, src/sDbscan.cpp), compiled against the shim headers
// in oracle/shim.  Test infrastructure only: it is built on the development
// machine (the reference sources are not present elsewhere) and used to pin
// the oracle restatement and to generate the golden fixtures in tests/golden.
//
// The probe subclasses sDbscan to read its protected state after a fit:
// matrix_topK / matrix_topM (src/sDbscan.h:50-51), bit_CorePoints (:56),
// vec2D_Neighbors (:54), vec2D_NeighborDist (:59), vec_CoreDist (:60),
// bitHD3 (:42) and matrix_R (:48).
#include "sDbscan.h"
#include "Utilities.h"

#include <cstdint>
#include <cstring>

namespace {

class RefProbe : public sDbscan {
public:
    RefProbe(int n, int d) : sDbscan(n, d) {}

    const MatrixXi& topK() const { return matrix_topK; }
    const MatrixXi& topM() const { return matrix_topM; }
    const boost::dynamic_bitset<>& core() const { return bit_CorePoints; }
    const vector<IVector>& neighbors() const { return vec2D_Neighbors; }
    const vector<vector<pair<int, float>>>& neighborDist() const { return vec2D_NeighborDist; }
    const FVector& coreDist() const { return vec_CoreDist; }
    const boost::dynamic_bitset<>& bits() const { return bitHD3; }
    const MatrixXf& R() const { return matrix_R; }
    int nProj() const { return n_proj; }
    int kerDim() const { return ker_n_features; }
    int nFeatures() const { return n_features; }
    int nPoints() const { return n_points; }
    const string& dist() const { return distance; }
    float kerSam() const { return ker_intervalSampling; }
    void setOutput(const char* prefix) { output = prefix; }

    // Projection of every (already transformed) point exactly as
    // src/sDbscan.cpp:53-91 forms MATRIX_FHT, using the fitted bitHD3 / matrix_R
    // and the reference's own fht_float.  Written here because MATRIX_FHT is a
    // local of the private rp_parIndex.
    void project(float* out) const {
        const int fhtDim = 1 << int(ceil(log2(max(n_proj, ker_n_features))));
        const int log2Project = log2(fhtDim);
        const int D = ker_n_features / 2;
        for (int n = 0; n < n_points; ++n) {
            VectorXf vecX = matrix_X.col(n);
            VectorXf vecEmbed = VectorXf::Zero(ker_n_features);
            if (distance == "Cosine")
                vecEmbed.segment(0, n_features) = vecX;
            else if (distance == "L1" || distance == "L2") {
                VectorXf vecProject = matrix_R * vecX;
                vecEmbed.segment(0, D) = vecProject.array().cos();
                vecEmbed.segment(D, D) = vecProject.array().sin();
            } else if (distance == "Chi2")
                embedChi2(vecX, ker_n_features, n_features, ker_intervalSampling, vecEmbed);
            else if (distance == "JS")
                embedJS(vecX, ker_n_features, n_features, ker_intervalSampling, vecEmbed);
            VectorXf rot = VectorXf::Zero(fhtDim);
            rot.segment(0, ker_n_features) = vecEmbed;
            for (int r = 0; r < 3; ++r) {
                for (int d = 0; d < fhtDim; ++d) rot(d) *= (2 * (int)bitHD3[r * fhtDim + d] - 1);
                fht_float(rot.data(), log2Project);
            }
            std::memcpy(out + (size_t)n * n_proj, rot.data(), sizeof(float) * n_proj);
        }
    }
};

RefProbe* P(void* h) { return static_cast<RefProbe*>(h); }

}  // namespace

extern "C" {

void* ref_new(int n, int d) { return new RefProbe(n, d); }
void ref_free(void* h) { delete P(h); }

// sDbscan::set_params (src/sDbscan.h:79-108), positional order kept.
void ref_set_params(void* h, int numProj, int k, int m, const char* dist, int kerDim, float kerSigma,
                    float kerSam, int noise, float prob, int verbose, int threads, int seed) {
    P(h)->set_params(numProj, k, m, string(dist), kerDim, kerSigma, kerSam, noise, prob, verbose != 0, "",
                     threads, seed);
}

// X is d x n column-major (one point per contiguous column), as the reference takes it.
void ref_fit_sdbscan(void* h, const float* X, int n, int d, float eps, int minPts) {
    Ref<const MatrixXf> ref(X, d, n);
    P(h)->fit_sDbscan(ref, eps, minPts);
}
void ref_fit_soptics(void* h, const float* X, int n, int d, float eps, int minPts) {
    Ref<const MatrixXf> ref(X, d, n);
    P(h)->fit_sOptics(ref, eps, minPts);
}
// sDbscan::set_sngParams (src/sDbscan.h:127-139), positional order kept.
void ref_set_sng_params(void* h, const char* dist, float prob, int noise, int verbose, int threads, int seed) {
    P(h)->set_sngParams(string(dist), prob, noise, verbose != 0, "", threads, seed);
}
void ref_fit_sngdbscan(void* h, const float* X, int n, int d, float eps, int minPts) {
    Ref<const MatrixXf> ref(X, d, n);
    P(h)->fit_sngDbscan(ref, eps, minPts);
}
void ref_fit_sngoptics(void* h, const float* X, int n, int d, float eps, int minPts) {
    Ref<const MatrixXf> ref(X, d, n);
    P(h)->fit_sngOptics(ref, eps, minPts);
}
// test_sDbscan (src/sDbscan.cpp:980-1039): index once, then one labels file
// per eps = eps + i * rangeEps, named from the output prefix.
void ref_test_sdbscan(void* h, const float* X, int n, int d, float eps, float rangeEps, int nTests, int minPts,
                      const char* prefix) {
    Ref<const MatrixXf> ref(X, d, n);
    P(h)->setOutput(prefix);
    P(h)->test_sDbscan(ref, eps, rangeEps, nTests, minPts);
}
// loadtxtData (src/Utilities.cpp:60-95) with distance "L2", which leaves the
// parsed values untransformed; out: n x d, one point per row.
void ref_load_txt(const char* path, int n, int d, float* out) {
    MatrixXf M;
    loadtxtData(string(path), "L2", n, d, M);
    std::memcpy(out, M.data(), sizeof(float) * (size_t)n * d);
}
void ref_clear(void* h) { P(h)->clear(); }

int ref_n_clusters(void* h) { return P(h)->n_clusters_; }
void ref_labels(void* h, int* out) { std::copy(P(h)->labels_.begin(), P(h)->labels_.end(), out); }
int64_t ref_ordering_size(void* h) { return (int64_t)P(h)->ordering_.size(); }
void ref_ordering(void* h, int* out) { std::copy(P(h)->ordering_.begin(), P(h)->ordering_.end(), out); }
void ref_reachability(void* h, float* out) {
    std::copy(P(h)->reachability_.begin(), P(h)->reachability_.end(), out);
}
void ref_topk(void* h, int* out) {
    const MatrixXi& t = P(h)->topK();
    std::memcpy(out, t.data(), sizeof(int) * t.size());
}
void ref_topm(void* h, int* out) {
    const MatrixXi& t = P(h)->topM();
    std::memcpy(out, t.data(), sizeof(int) * t.size());
}
void ref_core(void* h, uint8_t* out) {
    const auto& b = P(h)->core();
    for (size_t i = 0; i < b.size(); ++i) out[i] = b[i] ? 1 : 0;
}
void ref_core_dist(void* h, float* out) { std::copy(P(h)->coreDist().begin(), P(h)->coreDist().end(), out); }
int ref_bits_size(void* h) { return (int)P(h)->bits().size(); }
void ref_bits(void* h, uint8_t* out) {
    const auto& b = P(h)->bits();
    for (size_t i = 0; i < b.size(); ++i) out[i] = b[i] ? 1 : 0;
}
int ref_R_rows(void* h) { return (int)P(h)->R().rows(); }
int ref_R_cols(void* h) { return (int)P(h)->R().cols(); }
void ref_R(void* h, float* out) {
    const MatrixXf& R = P(h)->R();
    std::memcpy(out, R.data(), sizeof(float) * R.size());
}
void ref_matrix_X(void* h, float* out) {
    const MatrixXf& X = P(h)->matrix_X;
    std::memcpy(out, X.data(), sizeof(float) * X.size());
}
void ref_project(void* h, float* out) { P(h)->project(out); }

// Neighbour lists: sizes then the flattened lists (in the reference's order).
void ref_neighbor_sizes(void* h, int64_t* sizes) {
    const auto& v = P(h)->neighbors();
    for (size_t i = 0; i < v.size(); ++i) sizes[i] = (int64_t)v[i].size();
}
void ref_neighbors(void* h, int* flat) {
    size_t o = 0;
    for (const auto& l : P(h)->neighbors())
        for (int x : l) flat[o++] = x;
}
void ref_neighbor_dist_sizes(void* h, int64_t* sizes) {
    const auto& v = P(h)->neighborDist();
    for (size_t i = 0; i < v.size(); ++i) sizes[i] = (int64_t)v[i].size();
}
void ref_neighbor_dist(void* h, int* idx, float* dist) {
    size_t o = 0;
    for (const auto& l : P(h)->neighborDist())
        for (const auto& pr : l) {
            idx[o] = pr.first;
            dist[o] = pr.second;
            ++o;
        }
}

}  // extern "C"
