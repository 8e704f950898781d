// Host C++ class with the public API of the reference's `sDbscan`
// (src/sDbscan.h:62-201): same method names, argument order, defaults and
// public result members.  Compute runs on the GPU through the C ABI of
// include/sdbscan_gb300.h.
//
// Differences from the reference, all at the edges of the fit path:
//  - X is passed as a pointer to d x n column-major float data (the layout
//    Eigen::Ref<const MatrixXf> carries) instead of an Eigen reference;
//  - invalid input throws std::runtime_error where the reference prints and
//    calls exit(1) (src/Utilities.h:308-324);
//  - clusterNoise = 1 (sDbscan-1NN) samples core points with a seeded rule
//    instead of the reference's unseeded rand(); every core point is taken
//    when samplingProb n exceeds their number, as in the reference.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "sdbscan_gb300.h"

typedef std::vector<float> FVector;
typedef std::vector<int> IVector;

class sDbscan {
public:
    // Dbscan's output (src/sDbscan.h:67-68)
    IVector labels_;
    int n_clusters_ = 0;
    // Optics's output (src/sDbscan.h:71-72)
    IVector ordering_;
    FVector reachability_;

    sDbscan(int n, int d, int device = 0);
    ~sDbscan();
    sDbscan(const sDbscan&) = delete;
    sDbscan& operator=(const sDbscan&) = delete;

    // src/sDbscan.h:79-108
    void set_params(int numProj = 1024, int k = 5, int m = 50, std::string dist = "Cosine", int kerDim = 1024,
                    float kerSigma = 1.0, float kerSam = 0.4, int noiseClustering = 0, float prob = 0.01,
                    bool ver = false, std::string filename = "", int numThreads = 8, int randomSeed = -1);
    // src/sDbscan.h:110-124
    void set_kernel_params(std::string dist = "L2", int kerDim = 1024, float kerSigma = 1.0, float kerSam = 0.4);
    // src/sDbscan.h:142-163
    void clear();
    // src/sDbscan.h:170-180
    void set_topM(int m);
    void set_topK(int k);
    void set_proj(int p);
    void set_clusterNoise(int c);
    void set_threads(int t);
    // This engine's addition: SDB_PREC_FP32 (default) or SDB_PREC_BF16.
    void set_precision(int precision);

    // src/sDbscan.h:183 / src/sDbscan.cpp:830-890
    void fit_sDbscan(const float* X_dxn, float eps, int minPts);
    // src/sDbscan.h:197 / src/sDbscan.cpp:1711-1769
    void fit_sOptics(const float* X_dxn, float eps, int minPts);
    // load_fit_sDbscan / load_fit_sOptics (src/sDbscan.h:184, :198): the data
    // from a text file of n_points lines of n_features numbers, then the fit
    void load_fit_sDbscan(const std::string& dataset, float eps, int minPts);
    void load_fit_sOptics(const std::string& dataset, float eps, int minPts);
    // test_sDbscan / load_test_sDbscan (src/sDbscan.h:187-188): index once,
    // then a clustering for eps + i rangeEps (i < n_tests), each written to
    // its labels file; labels_ keeps the last one
    void test_sDbscan(const float* X_dxn, float eps, float rangeEps, int n_tests, int minPts);
    void load_test_sDbscan(const std::string& dataset, float eps, float rangeEps, int n_tests, int minPts);

    // sngDbscan / sngOptics (src/sDbscan.h:127-139, :190-201): the sampled
    // neighbourhood baselines.  With randomSeed >= 0, fit_sngDbscan's labels
    // equal the reference's; sngOptics shares one seeded sample across points
    // where the reference draws each point's from std::random_device.
    void set_sngParams(std::string dist = "Cosine", float prob = 0.01, int noiseClustering = 0, bool ver = false,
                       std::string filename = "", int numThreads = -1, int randomSeed = -1);
    void fit_sngDbscan(const float* X_dxn, float eps, int minPts);
    void test_sngDbscan(const float* X_dxn, float eps, float rangeEps, int n_tests, int minPts);
    void load_test_sngDbscan(const std::string& dataset, float eps, float rangeEps, int n_tests, int minPts);
    void fit_sngOptics(const float* X_dxn, float eps, int minPts);
    void load_fit_sngOptics(const std::string& dataset, float eps, int minPts);

    int n_points() const { return n_; }
    int n_features() const { return d_; }
    sdb_engine* engine() { return eng_; }

private:
    void push_params();
    std::string sng_file(float eps, int minPts) const;
    void check(sdb_status s, const char* what);
    int n_, d_;
    sdb_params prm_;
    std::string output_;
    sdb_engine* eng_ = nullptr;
};
