// Operators on SO(3) coefficients and harmonics, on the GPU: directional
// derivatives of an SO(3) function and Clebsch-Gordan tables.
//
// Derivative.  With d/dt D^l(R exp(t e_i)) |_{t=0} = D^l(R) u_i^l
// (deriv_wigner_D, fdcl_FFTSO3.cpp:417-453; for the real harmonics
// d/dt U^l(R exp(t e_i)) = U^l(R) u_i^l, deriv_real_harmonics, :1577-1645), the
// function f(R) = sum_l (2l+1) sum_mn F^l_mn D^l_mn(R) has the derivative
// f_i(R) = d/dt f(R exp(t e_i)) with coefficients F'^l = F^l (u_i^l)^T.  Every
// row of u_i^l has at most two nonzeros, so each output coefficient is a
// two-term sum over one row of the per-plan table of (column, value) pairs.
//
// Clebsch-Gordan.  For fixed (l1, l2) the coefficients form the orthogonal
// matrix C of src/fdcl_Clebsch_Gordon.cpp (row (l1+m1)(2l2+1) + l2 + m2, column
// l^2 - (l2-l1)^2 + l + m, :18-26), D^{l1} (x) D^{l2} = C ((+)_l D^l) C^T.  Each
// column (l, m) is the solution of the three-term relation in m1 that the
// reference solves in compute_sub (:41-84, after Straub 2014): started at the
// largest m1 with 1, run down, normalised (so the largest-m1 entry stays
// positive) -- one GPU thread per column.  The real-harmonic coefficients
// c = conj(T^{l1} (x) T^{l2}) C ((+)_l T^l)^T (:224-329, T = matrix2rsph) take
// one thread per entry: every row of T has at most two nonzeros, so each entry
// of c is a sum of at most 8 products of C.
#include <cmath>

#include "common.cuh"
#include "operators.cuh"
#include "rsph.cuh"

namespace fftso3 {

namespace {

// l of packed index i (so3_off(l) <= i < so3_off(l + 1))
__device__ __forceinline__ int packed_l(long long i)
{
    int l = (int)cbrt(0.75 * (double)i);
    while (l > 0 && so3_off(l) > i) --l;
    while (so3_off(l + 1) <= i) ++l;
    return l;
}

// T the element type (complex or real), A its arithmetic (double for FP64 plans, float otherwise)
template <typename T, typename A, bool CPLX>
__global__ void derivative_kernel(const T* __restrict__ F, T* __restrict__ out, const DerivEntry* __restrict__ tab,
                                  int L, long long C, long long total)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long f = idx / C, i = idx - f * C;
    const int l = packed_l(i);
    const int W = 2 * l + 1;
    const long long r = i - so3_off(l);
    const int mi = (int)(r % W), ki = (int)(r / W);  // F(m, k) at (m + l) + (k + l) W
    const DerivEntry e = tab[(long long)l * l + ki];  // row k of u_i^l
    const long long base = f * C + so3_off(l) + mi;
    if constexpr (CPLX) {
        A ax = 0, ay = 0;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (e.col[j] < 0) continue;
            const T v = F[base + (long long)e.col[j] * W];
            const A ur = (A)e.re[j], ui = (A)e.im[j];
            ax += ur * v.x - ui * v.y;
            ay += ur * v.y + ui * v.x;
        }
        T o;
        o.x = ax;
        o.y = ay;
        out[idx] = o;
    } else {
        A a = 0;
#pragma unroll
        for (int j = 0; j < 2; ++j)
            if (e.col[j] >= 0) a += (A)e.re[j] * F[base + (long long)e.col[j] * W];
        out[idx] = a;
    }
}

// One thread per column (l, m) of C (n x n, column-major, zeroed by the caller).
__global__ void cg_columns_kernel(int l1, int l2, double* __restrict__ C, long long n)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int lmin = l1 > l2 ? l1 - l2 : l2 - l1;
    const long long q = c + (long long)lmin * lmin;  // l^2 + l + m
    int l = (int)sqrt((double)q);
    while ((long long)l * l > q) --l;
    while ((long long)(l + 1) * (l + 1) <= q) ++l;
    const int m = (int)(q - (long long)l * l - l);
    const int lo = max(-l1, m - l2), hi = min(l1, m + l2);
    if (lo > hi) return;
    const double a1 = l1 * (l1 + 1.0), a2 = l2 * (l2 + 1.0), al = l * (l + 1.0);
    auto diag = [&](int m1) { return a1 + a2 + 2.0 * m1 * (m - m1) - al; };
    auto off = [&](int m1) {  // coupling of m1 and m1 - 1
        const int m2 = m - m1;
        return sqrt((a1 - m1 * (m1 - 1.0)) * (a2 - m2 * (m2 + 1.0)));
    };
    double* col = C + c * n;
    auto row = [&](int m1) { return (long long)(l1 + m1) * (2 * l2 + 1) + l2 + (m - m1); };
    // run down from c(hi) = 1 (c(hi + 1) = 0), writing the unnormalised values
    double cur = 1.0, above = 0.0, nrm = 1.0;
    col[row(hi)] = 1.0;
    for (int m1 = hi; m1 > lo; --m1) {
        const double below = -(diag(m1) * cur + off(m1 + 1) * above) / off(m1);
        col[row(m1 - 1)] = below;
        nrm += below * below;
        above = cur;
        cur = below;
    }
    const double s = 1.0 / sqrt(nrm);
    for (int m1 = lo; m1 <= hi; ++m1) col[row(m1)] *= s;
}

// c = conj(T^{l1} (x) T^{l2}) C O^T, O = (+)_l T^l; one thread per entry (row, col), complex output.
__global__ void cg_real_kernel(int l1, int l2, const double* __restrict__ C, double2* __restrict__ out, long long n)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * n) return;
    const long long col = e / n, row = e - col * n;  // column-major
    const int W2 = 2 * l2 + 1;
    const int a1 = (int)(row / W2) - l1, a2 = (int)(row % W2) - l2;  // row of T1 (x) T2
    const int lmin = l1 > l2 ? l1 - l2 : l2 - l1;
    const long long q = col + (long long)lmin * lmin;
    int l = (int)sqrt((double)q);
    while ((long long)l * l > q) --l;
    while ((long long)(l + 1) * (l + 1) <= q) ++l;
    const int a = (int)(q - (long long)l * l - l);  // row of T^l
    const long long cbase = (long long)l * l - (long long)lmin * lmin + l;  // column index of (l, 0)
    // the nonzero columns of row a1 of T1, a2 of T2, a of T^l: c and -c
    int c1[2] = {a1, -a1}, c2[2] = {a2, -a2}, c3[2] = {a, -a};
    const int n1 = a1 == 0 ? 1 : 2, n2 = a2 == 0 ? 1 : 2, n3 = a == 0 ? 1 : 2;
    double sx = 0.0, sy = 0.0;
    for (int i = 0; i < n1; ++i) {
        const c2t<double> t1 = conj_t(tmat_t<double>(a1, c1[i]));
        for (int j = 0; j < n2; ++j) {
            const c2t<double> t12 = cmul_t(t1, conj_t(tmat_t<double>(a2, c2[j])));
            const long long r2 = (long long)(l1 + c1[i]) * W2 + l2 + c2[j];
            for (int k = 0; k < n3; ++k) {
                const c2t<double> t3 = tmat_t<double>(a, c3[k]);
                const double v = C[(cbase + c3[k]) * n + r2];
                const c2t<double> p = cmul_t(t12, t3);
                sx += p.x * v;
                sy += p.y * v;
            }
        }
    }
    out[e] = make_double2(sx, sy);
}

}  // namespace

// Rows of u_i^l, l <= L (table [3][(L+1)^2]: row l^2 + k + l, k = -l..l), from the formulas of
// fdcl_FFTSO3.cpp:417-453 (complex harmonics) or :1577-1645 (real harmonics).
std::vector<DerivEntry> derivative_table(int L, bool real)
{
    const long long R = (long long)(L + 1) * (L + 1);
    std::vector<DerivEntry> t(3 * R);
    for (auto& e : t) {
        e.col[0] = e.col[1] = -1;
        e.re[0] = e.re[1] = e.im[0] = e.im[1] = 0.0;
    }
    bool over = false;  // a third nonzero in one row (the formulas give at most two)
    auto add = [&](int axis, int l, int k, int n, double re, double im) {
        DerivEntry& e = t[(axis - 1) * R + (long long)l * l + k + l];
        if (e.col[1] >= 0) over = true;
        const int j = e.col[0] < 0 ? 0 : 1;
        e.col[j] = n + l;
        e.re[j] = re;
        e.im[j] = im;
    };
    for (int l = 0; l <= L; ++l) {
        if (!real) {
            for (int k = -l; k <= l; ++k) {
                if (k != 0) add(3, l, k, k, 0.0, -(double)k);
                if (k < l) {
                    const double c = sqrt((l + k + 1.0) * (l - k));
                    add(2, l, k, k + 1, 0.5 * c, 0.0);
                    add(1, l, k, k + 1, 0.0, -0.5 * c);
                }
                if (k > -l) {
                    const double c = sqrt((l - k + 1.0) * (l + k));
                    add(2, l, k, k - 1, -0.5 * c, 0.0);
                    add(1, l, k, k - 1, 0.0, -0.5 * c);
                }
            }
        } else {
            for (int p = 1; p <= l; ++p) {
                add(3, l, p, -p, -(double)p, 0.0);
                add(3, l, -p, p, (double)p, 0.0);
            }
            for (int p = 2; p <= l; ++p) {
                const double s = 0.5 * sqrt((l + p) * (l - p + 1.0));
                add(2, l, p, p - 1, s, 0.0);
                add(2, l, -p, -p + 1, s, 0.0);
                add(1, l, p, -p + 1, s, 0.0);
                add(1, l, -p, p - 1, -s, 0.0);
                const int q = p - 1;
                const double u = 0.5 * sqrt((l - q) * (l + q + 1.0));
                add(2, l, q, q + 1, -u, 0.0);
                add(2, l, -q, -q - 1, -u, 0.0);
                add(1, l, q, -q - 1, u, 0.0);
                add(1, l, -q, q + 1, -u, 0.0);
            }
            if (l >= 1) {
                const double s = sqrt(l * (l + 1.0) / 2.0);
                add(2, l, 1, 0, s, 0.0);
                add(2, l, 0, 1, -s, 0.0);
                add(1, l, -1, 0, -s, 0.0);
                add(1, l, 0, -1, s, 0.0);
            }
        }
    }
    if (over) t.clear();
    return t;
}

cudaError_t launch_derivative(const void* F, void* out, const DerivEntry* tab, bool fp64, bool real, int L,
                              int batch, cudaStream_t st)
{
    const long long C = so3_off(L + 1), total = C * batch;
    const unsigned nb = (unsigned)((total + 255) / 256);
    if (fp64 && !real)
        derivative_kernel<double2, double, true><<<nb, 256, 0, st>>>((const double2*)F, (double2*)out, tab, L, C, total);
    else if (fp64)
        derivative_kernel<double, double, false><<<nb, 256, 0, st>>>((const double*)F, (double*)out, tab, L, C, total);
    else if (!real)
        derivative_kernel<float2, float, true><<<nb, 256, 0, st>>>((const float2*)F, (float2*)out, tab, L, C, total);
    else
        derivative_kernel<float, float, false><<<nb, 256, 0, st>>>((const float*)F, (float*)out, tab, L, C, total);
    return cudaGetLastError();
}

cudaError_t launch_clebsch_gordan(int l1, int l2, double* C, double2* creal, cudaStream_t st)
{
    const long long n = (long long)(2 * l1 + 1) * (2 * l2 + 1);
    cudaError_t e = cudaMemsetAsync(C, 0, sizeof(double) * n * n, st);
    if (e != cudaSuccess) return e;
    cg_columns_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(l1, l2, C, n);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (creal) {
        cg_real_kernel<<<(unsigned)((n * n + 255) / 256), 256, 0, st>>>(l1, l2, C, creal, n);
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace fftso3
