// Shared device/host helpers for the GB300 SO(3)/S^2 transform library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace fftso3 {

// Packed SO(3) coefficient layout (fdcl_FFTSO3_matrix.cpp:43-47 stores
// M[l](m+l, n+l) column-major): off(l) = l(4l^2-1)/3.
__host__ __device__ __forceinline__ long long so3_off(int l) { return (long long)l * (4LL * l * l - 1) / 3; }
__host__ __device__ __forceinline__ long long so3_idx(int l, int m, int n) {
    return so3_off(l) + (m + l) + (long long)(n + l) * (2 * l + 1);
}
// Packed S^2 layout (fdcl_FFTS2_matrix.cpp:43-47): l^2 + m + l.
__host__ __device__ __forceinline__ long long s2_idx(int l, int m) { return (long long)l * l + m + l; }

// Symmetry group of the Wigner-d table.  Group g <-> (m0, n0) with m0 >= |n0|,
// g = m0^2 + m0 + n0.  The table stores d^l_{m0 n0}(beta_k) for l = m0..L; the
// other members of the orbit use it with a sign (fdcl_FFTSO3.cpp:173-190):
//   (m0,n0): +1   (-m0,-n0): (-1)^(m0+n0)   (n0,m0): (-1)^(m0+n0)   (-n0,-m0): +1
struct GroupPairs {
    int np;        // number of distinct (m,n) pairs served by the group (1, 2 or 4)
    int m[4], n[4];
    int sign[4];   // +1 or -1
};

__host__ __device__ __forceinline__ void group_mn(int g, int& m0, int& n0) {
    int m = (int)sqrtf((float)g);
    while (m * m > g) --m;
    while ((m + 1) * (m + 1) <= g) ++m;
    m0 = m;
    n0 = g - m * m - m;
}

__host__ __device__ __forceinline__ GroupPairs group_pairs(int m0, int n0) {
    GroupPairs p;
    const int s = ((m0 + n0) & 1) ? -1 : 1;
    p.m[0] = m0;  p.n[0] = n0;  p.sign[0] = 1;
    if (m0 == 0) { p.np = 1; return p; }
    p.m[1] = -m0; p.n[1] = -n0; p.sign[1] = s;
    if (n0 == m0 || n0 == -m0) { p.np = 2; return p; }
    p.m[2] = n0;  p.n[2] = m0;  p.sign[2] = s;
    p.m[3] = -n0; p.n[3] = -m0; p.sign[3] = 1;
    p.np = 4;
    return p;
}

// (m, n) -> (symmetry group g, pair p) consistent with group_pairs(): m0 = max(|m|, |n|), g = m0^2 + m0 + n0.
__host__ __device__ __forceinline__ void pair_of(int m, int n, int& g, int& p) {
    int m0, n0;
    const int am = m < 0 ? -m : m, an = n < 0 ? -n : n;
    if (am >= an) {
        if (m >= 0) { m0 = m; n0 = n; p = 0; }
        else { m0 = -m; n0 = -n; p = 1; }
    } else {
        if (n > 0) { m0 = n; n0 = m; p = 2; }
        else { m0 = -n; n0 = -m; p = 3; }
    }
    g = m0 * m0 + m0 + n0;
}

// Records the message returned by fftso3_last_error_string() on this thread.
void set_last_error(const std::string& msg);

template <typename T> struct cplx;
template <> struct cplx<double> { using type = double2; };
template <> struct cplx<float> { using type = float2; };

}  // namespace fftso3
