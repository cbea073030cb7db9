/*
 * ref_naive_shim.cpp -- builds the reference's own CPU k-means
 * (kmeans_naive.cpp, kmeans_initializer.cpp, matrix.hpp) unchanged, from where
 * its sources lie, and exposes it through a small C ABI for the tests.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle's pin).  Built by oracle/build_ref.sh
 * into oracle/_ref/ when the reference tree is present; never part of the
 * product library.
 *
 * The reference header measurement/measurement.hpp needs Boost.Compute.
 * KmeansNaive only constructs an empty Measurement, so this file defines the
 * header's include guard and a one-class stand-in before the reference
 * sources are included.
 */
#define MEASUREMENT_HPP
#include <memory>
namespace Measurement { class Measurement {}; }

#include "kmeans_naive.cpp"
#include "kmeans_initializer.cpp"

#include <chrono>
#include <cstring>

namespace {
template <typename T>
cle::Matrix<T, std::allocator<T>, size_t, true> make_matrix(T const* data, size_t rows, size_t cols) {
    cle::Matrix<T, std::allocator<T>, size_t, true> m;
    m.resize(rows, cols);
    std::memcpy(&*m.begin(), data, sizeof(T) * rows * cols);
    return m;
}

template <typename PointT, typename LabelT, typename MassT>
int run_naive(PointT const* points, uint64_t n, uint32_t d, uint32_t k, uint32_t iterations,
              PointT* centroids, MassT* masses, LabelT* labels, int init_first_x,
              uint64_t* loop_ns = nullptr) {
    auto P = make_matrix(points, n, d);
    cle::Matrix<PointT, std::allocator<PointT>, size_t, true> C;
    C.resize(k, d);
    if (init_first_x) {
        Clustering::KmeansInitializer<PointT>::first_x(P, C);
    } else {
        std::memcpy(&*C.begin(), centroids, sizeof(PointT) * k * d);
    }
    std::vector<MassT> M(k, 0);
    std::vector<LabelT> L(n, 0);
    Clustering::KmeansNaive<PointT, LabelT, MassT> naive;
    naive.initialize();
    auto t0 = std::chrono::steady_clock::now();
    naive(iterations, P, C, M, L);
    auto t1 = std::chrono::steady_clock::now();
    naive.finalize();
    if (loop_ns)
        *loop_ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count();
    std::memcpy(centroids, &*C.begin(), sizeof(PointT) * k * d);
    std::memcpy(masses, M.data(), sizeof(MassT) * k);
    std::memcpy(labels, L.data(), sizeof(LabelT) * n);
    return 0;
}
}

extern "C" {

/* KmeansNaive32 (kmeans_naive.hpp:39-40) over column-major points.  When
 * init_first_x is set, the centroids are first set by
 * KmeansInitializer::first_x (kmeans_initializer.cpp:29-39). */
int ckm_ref_naive_f32(float const* points, uint64_t n, uint32_t d, uint32_t k,
                      uint32_t iterations, float* centroids, uint32_t* masses,
                      uint32_t* labels, int init_first_x) {
    return run_naive<float, uint32_t, uint32_t>(points, n, d, k, iterations, centroids,
                                                masses, labels, init_first_x);
}

/* The same call, also returning the wall time of the KmeansNaive call alone
 * (the iteration loop, kmeans_naive.cpp:31-106), without the copies into and
 * out of the reference's Matrix type.  Timed CPU baseline of bench.py. */
int ckm_ref_naive_f32_timed(float const* points, uint64_t n, uint32_t d, uint32_t k,
                            uint32_t iterations, float* centroids, uint32_t* masses,
                            uint32_t* labels, int init_first_x, uint64_t* loop_ns) {
    return run_naive<float, uint32_t, uint32_t>(points, n, d, k, iterations, centroids,
                                                masses, labels, init_first_x, loop_ns);
}

/* KmeansNaive64 (kmeans_naive.hpp:41-42). */
int ckm_ref_naive_f64(double const* points, uint64_t n, uint32_t d, uint32_t k,
                      uint32_t iterations, double* centroids, uint64_t* masses,
                      uint64_t* labels, int init_first_x) {
    return run_naive<double, uint64_t, uint64_t>(points, n, d, k, iterations, centroids,
                                                 masses, labels, init_first_x);
}

}
