// The CPU reference of `ckm_bench --verify` (the reference's --verify pass,
// clustering_benchmark.cpp:276-326, compares against KmeansNaive): a
// single-threaded Lloyd with the arithmetic of kmeans_naive.cpp:40-103 --
// fma distance, strict '<' argmin from the type's maximum with label 0, Kahan
// sums, 0/0 -> NaN means.  Column-major points P[f * n + p] and centroids
// C[f * k + c]; C holds the initial centroids on entry and the result on exit.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

template <typename P, typename L, typename M>
void verify_naive(uint32_t iterations, const std::vector<P>& pts, size_t n, size_t d, std::vector<P>& C,
                  std::vector<M>& masses, std::vector<L>& labels) {
    const size_t k = C.size() / d;
    std::vector<P> comp(k * d);
    for (uint32_t it = 0; it < iterations; ++it) {
        for (size_t p = 0; p < n; ++p) {
            P best = std::numeric_limits<P>::max();
            L lab = 0;
            for (size_t c = 0; c < k; ++c) {
                P dist = 0;
                for (size_t f = 0; f < d; ++f) {
                    P t = pts[f * n + p] - C[f * k + c];
                    dist = std::fma(t, t, dist);
                }
                if (dist < best) {
                    best = dist;
                    lab = (L)c;
                }
            }
            labels[p] = lab;
        }
        std::fill(masses.begin(), masses.end(), 0);
        std::fill(C.begin(), C.end(), 0);
        std::fill(comp.begin(), comp.end(), 0);
        for (size_t p = 0; p < n; ++p) {
            const L c = labels[p];
            masses[c] += 1;
            for (size_t f = 0; f < d; ++f) {
                P& s = C[f * k + c];
                P& cp = comp[f * k + c];
                volatile P y = pts[f * n + p] - cp;
                volatile P t = s + y;
                cp = (t - s) - y;
                s = t;
            }
        }
        for (size_t f = 0; f < d; ++f)
            for (size_t c = 0; c < k; ++c) C[f * k + c] = C[f * k + c] / (P)masses[c];
    }
}

