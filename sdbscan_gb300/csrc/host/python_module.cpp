// Python module `sDbscan` with the names, keyword arguments and defaults of
// the reference binding (python/python_wrapper.cpp:14-65), over the host
// class of sDbscan.h.  X is a float32 array of shape (n_features, n_points),
// as in the reference (README.md:39-41); it is read column-major.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include "sDbscan.h"

namespace py = pybind11;

namespace {

using FArray = py::array_t<float, py::array::f_style | py::array::forcecast>;

const float* checked(sDbscan& s, const FArray& X) {
    if (X.ndim() != 2 || X.shape(0) != s.n_features() || X.shape(1) != s.n_points())
        throw std::invalid_argument("X must have shape (n_features, n_points) = (" + std::to_string(s.n_features()) +
                                    ", " + std::to_string(s.n_points()) + ")");
    return X.data();
}

}  // namespace

PYBIND11_MODULE(sDbscan, m) {
    py::class_<sDbscan>(m, "sDbscan")
        .def(py::init<int, int, int>(), py::arg("n_points"), py::arg("n_features"), py::arg("device") = 0)
        .def("set_params", &sDbscan::set_params, py::arg("n_proj") = 1024, py::arg("topK") = 10,
             py::arg("topM") = 50, py::arg("distance") = "Cosine", py::arg("ker_n_features") = 1024,
             py::arg("ker_sigma") = 1.0, py::arg("ker_intervalSampling") = 0.4, py::arg("clusterNoise") = 0,
             py::arg("samplingProb") = 0.01, py::arg("verbose") = false, py::arg("output") = "",
             py::arg("n_threads") = -1, py::arg("random_seed") = -1)
        .def_readonly("labels_", &sDbscan::labels_)
        .def_readonly("n_clusters_", &sDbscan::n_clusters_)
        .def_readonly("ordering_", &sDbscan::ordering_)
        .def_readonly("reachability_", &sDbscan::reachability_)
        .def("clear", &sDbscan::clear)
        .def("set_topM", &sDbscan::set_topM, py::arg("topM"))
        .def("set_threads", &sDbscan::set_threads, py::arg("n_threads"))
        .def("set_clusterNoise", &sDbscan::set_clusterNoise, py::arg("clusterNoise"))
        .def("set_topK", &sDbscan::set_topK, py::arg("topK"))
        .def("set_kernel_params", &sDbscan::set_kernel_params, py::arg("distance") = "L2",
             py::arg("ker_n_features") = 1024, py::arg("ker_sigma") = 1.0, py::arg("ker_intervalSampling") = 0.4)
        .def("set_precision", &sDbscan::set_precision, py::arg("precision"))
        .def(
            "fit_sDbscan",
            [](sDbscan& s, const FArray& X, float eps, int minPts) {
                const float* p = checked(s, X);
                py::gil_scoped_release nogil;
                s.fit_sDbscan(p, eps, minPts);
            },
            py::arg("X"), py::arg("eps"), py::arg("minPts"))
        .def(
            "fit_sOptics",
            [](sDbscan& s, const FArray& X, float eps, int minPts) {
                const float* p = checked(s, X);
                py::gil_scoped_release nogil;
                s.fit_sOptics(p, eps, minPts);
            },
            py::arg("X"), py::arg("eps"), py::arg("minPts"))
        .def(
            "load_fit_sDbscan",
            [](sDbscan& s, const std::string& dataset, float eps, int minPts) {
                py::gil_scoped_release nogil;
                s.load_fit_sDbscan(dataset, eps, minPts);
            },
            py::arg("dataset"), py::arg("eps"), py::arg("minPts"))
        .def(
            "test_sDbscan",
            [](sDbscan& s, const FArray& X, float eps, float rangeEps, int n_tests, int minPts) {
                const float* p = checked(s, X);
                py::gil_scoped_release nogil;
                s.test_sDbscan(p, eps, rangeEps, n_tests, minPts);
            },
            py::arg("X"), py::arg("eps"), py::arg("rangeEps"), py::arg("n_tests"), py::arg("minPts"))
        .def(
            "load_test_sDbscan",
            [](sDbscan& s, const std::string& dataset, float eps, float rangeEps, int n_tests, int minPts) {
                py::gil_scoped_release nogil;
                s.load_test_sDbscan(dataset, eps, rangeEps, n_tests, minPts);
            },
            py::arg("dataset"), py::arg("eps"), py::arg("rangeEps"), py::arg("n_tests"), py::arg("minPts"))
        .def(
            "load_fit_sOptics",
            [](sDbscan& s, const std::string& dataset, float eps, int minPts) {
                py::gil_scoped_release nogil;
                s.load_fit_sOptics(dataset, eps, minPts);
            },
            py::arg("dataset"), py::arg("eps"), py::arg("minPts"))
        // sngDbscan / sngOptics (python/python_wrapper.cpp:26-27, :56-64)
        .def("set_sngParams", &sDbscan::set_sngParams, py::arg("distance") = "Cosine", py::arg("samplingProb") = 0.01,
             py::arg("clusterNoise") = 0, py::arg("verbose") = false, py::arg("output") = "",
             py::arg("n_threads") = -1, py::arg("random_seed") = -1)
        .def(
            "fit_sngDbscan",
            [](sDbscan& s, const FArray& X, float eps, int minPts) {
                const float* p = checked(s, X);
                py::gil_scoped_release nogil;
                s.fit_sngDbscan(p, eps, minPts);
            },
            py::arg("X"), py::arg("eps"), py::arg("minPts"))
        .def(
            "test_sngDbscan",
            [](sDbscan& s, const FArray& X, float eps, float rangeEps, int n_tests, int minPts) {
                const float* p = checked(s, X);
                py::gil_scoped_release nogil;
                s.test_sngDbscan(p, eps, rangeEps, n_tests, minPts);
            },
            py::arg("X"), py::arg("eps"), py::arg("rangeEps"), py::arg("n_tests"), py::arg("minPts"))
        .def(
            "load_test_sngDbscan",
            [](sDbscan& s, const std::string& dataset, float eps, float rangeEps, int n_tests, int minPts) {
                py::gil_scoped_release nogil;
                s.load_test_sngDbscan(dataset, eps, rangeEps, n_tests, minPts);
            },
            py::arg("dataset"), py::arg("eps"), py::arg("rangeEps"), py::arg("n_tests"), py::arg("minPts"))
        .def(
            "fit_sngOptics",
            [](sDbscan& s, const FArray& X, float eps, int minPts) {
                const float* p = checked(s, X);
                py::gil_scoped_release nogil;
                s.fit_sngOptics(p, eps, minPts);
            },
            py::arg("X"), py::arg("eps"), py::arg("minPts"))
        .def(
            "load_fit_sngOptics",
            [](sDbscan& s, const std::string& dataset, float eps, int minPts) {
                py::gil_scoped_release nogil;
                s.load_fit_sngOptics(dataset, eps, minPts);
            },
            py::arg("dataset"), py::arg("eps"), py::arg("minPts"));
}
