// C entry points over the reference's own transform classes, compiled unmodified from the reference's sources
// against the Eigen-API subset in ref_shim/ (recipe: ref.mk, output oracle/_ref/libfdcl_ref.so).  Test
// infrastructure only: it pins the restated oracle (fftso3_oracle.c) to the reference's actual code.
//
// Array conventions are the oracle's: SO(3) grid [k][j1][j2] = f(alpha_j1, beta_k, gamma_j2), S^2 grid
// [k][j] = f(theta_k, phi_j), complex values as interleaved (re, im) doubles; packed coefficients
// (l, m, n) at l(4l^2-1)/3 + (m+l) + (n+l)(2l+1) and (l, m) at l^2 + m + l.
//
// The reference's forward transforms take a callable f(alpha, beta, gamma) (fdcl_FFTSO3.hpp:76,232;
// fdcl_FFTS2.hpp:59,136) that they evaluate on the grid alpha_j = j pi / B, beta_k = (2k+1) pi / (4B)
// (fdcl_FFTSO3.cpp:578-591, fdcl_FFTS2.cpp:292-300); the callables here look the sample up by inverting those
// formulas, so the reference transforms exactly the given samples.
#include <cmath>
#include <complex>
#include <functional>
#include <stdexcept>

#include "fdcl_Clebsch_Gordon.hpp"
#include "fdcl_FFTS2.hpp"
#include "fdcl_FFTSO3.hpp"

namespace {

using cd = std::complex<double>;

inline long so3_idx(int l, int m, int n) { return (long)l * (4L * l * l - 1) / 3 + (m + l) + (long)(n + l) * (2 * l + 1); }
inline long s2_idx(int l, int m) { return (long)l * l + m + l; }

// grid index of an angle alpha_j = j pi / B (mod 2B) and of beta_k = (2k+1) pi / (4B)
inline int j_of(double a, int B)
{
    const int N = 2 * B;
    return (int)(((std::lround(a * B / M_PI) % N) + N) % N);
}
inline int k_of(double b, int B) { return (int)std::lround((b * 4.0 * B / M_PI - 1.0) / 2.0); }

template <typename T, typename M> void so3_unpack(int L, const T* src, M& F)
{
    for (int l = 0; l <= L; ++l)
        for (int m = -l; m <= l; ++m)
            for (int n = -l; n <= l; ++n) F(l, m, n) = src[so3_idx(l, m, n)];
}
template <typename T, typename M> void s2_unpack(int L, const T* src, M& F)
{
    for (int l = 0; l <= L; ++l)
        for (int m = -l; m <= l; ++m) F(l, m) = src[s2_idx(l, m)];
}

template <typename Fn> int guarded(Fn&& fn)
{
    try {
        fn();
        return 0;
    } catch (const std::exception&) {
        return 1;
    }
}

}  // namespace

extern "C" {

// fdcl::FFTSO3_complex::forward_transform (fdcl_FFTSO3.cpp:654-772): out = packed F, complex
int ref_so3_forward_complex(int L, const double* grid, double* out)
{
    return guarded([&] {
        const int B = L + 1, N = 2 * B;
        const cd* g = reinterpret_cast<const cd*>(grid);
        fdcl::FFTSO3_complex t(L);
        auto f = [&](double a, double b, double c) -> cd {
            return g[((long)k_of(b, B) * N + j_of(a, B)) * N + j_of(c, B)];
        };
        fdcl::FFTSO3_matrix_complex F = t.forward_transform(std::function<cd(double, double, double)>(f));
        cd* o = reinterpret_cast<cd*>(out);
        for (int l = 0; l <= L; ++l)
            for (int m = -l; m <= l; ++m)
                for (int n = -l; n <= l; ++n) o[so3_idx(l, m, n)] = F(l, m, n);
    });
}

// fdcl::FFTSO3_real::forward_transform (fdcl_FFTSO3.cpp:774-852): out = packed real F
int ref_so3_forward_real(int L, const double* grid, double* out)
{
    return guarded([&] {
        const int B = L + 1, N = 2 * B;
        fdcl::FFTSO3_real t(L);
        auto f = [&](double a, double b, double c) -> double {
            return grid[((long)k_of(b, B) * N + j_of(a, B)) * N + j_of(c, B)];
        };
        fdcl::FFTSO3_matrix_real F = t.forward_transform(std::function<double(double, double, double)>(f));
        for (int l = 0; l <= L; ++l)
            for (int m = -l; m <= l; ++m)
                for (int n = -l; n <= l; ++n) out[so3_idx(l, m, n)] = F(l, m, n);
    });
}

// fdcl::FFTSO3_complex::inverse_transform(F, alpha, beta, gamma) (fdcl_FFTSO3.cpp:498-576): out = (re, im)
int ref_so3_inverse_complex_point(int L, const double* coeffs, double a, double b, double c, double* out)
{
    return guarded([&] {
        fdcl::FFTSO3_complex t(L);
        fdcl::FFTSO3_matrix_complex F(L);
        so3_unpack(L, reinterpret_cast<const cd*>(coeffs), F);
        const cd v = t.inverse_transform(F, a, b, c);
        out[0] = v.real();
        out[1] = v.imag();
    });
}

// fdcl::FFTSO3_real::inverse_transform(F, alpha, beta, gamma)
int ref_so3_inverse_real_point(int L, const double* coeffs, double a, double b, double c, double* out)
{
    return guarded([&] {
        fdcl::FFTSO3_real t(L);
        fdcl::FFTSO3_matrix_real F(L);
        so3_unpack(L, coeffs, F);
        out[0] = t.inverse_transform(F, a, b, c);
    });
}

// fdcl::FFTSO3_complex::wigner_d(beta): packed d^l_mn(beta), l <= L
int ref_wigner_d(int L, double beta, double* out)
{
    return guarded([&] {
        fdcl::FFTSO3_complex t(L);
        fdcl::FFTSO3_matrix_real d = t.wigner_d(beta);
        for (int l = 0; l <= L; ++l)
            for (int m = -l; m <= l; ++m)
                for (int n = -l; n <= l; ++n) out[so3_idx(l, m, n)] = d(l, m, n);
    });
}

// fdcl::FFTSO3_real::real_harmonics(alpha, beta, gamma): packed U^l_mn
int ref_so3_real_harmonics(int L, double a, double b, double c, double* out)
{
    return guarded([&] {
        fdcl::FFTSO3_real t(L);
        fdcl::FFTSO3_matrix_real U = t.real_harmonics(a, b, c);
        for (int l = 0; l <= L; ++l)
            for (int m = -l; m <= l; ++m)
                for (int n = -l; n <= l; ++n) out[so3_idx(l, m, n)] = U(l, m, n);
    });
}

// fdcl::FFTS2_complex::forward_transform (fdcl_FFTS2.cpp:125-230): out = packed F, complex
int ref_s2_forward_complex(int L, const double* grid, double* out)
{
    return guarded([&] {
        const int B = L + 1, N = 2 * B;
        const cd* g = reinterpret_cast<const cd*>(grid);
        fdcl::FFTS2_complex t(L);
        auto f = [&](double th, double ph) -> cd { return g[(long)k_of(th, B) * N + j_of(ph, B)]; };
        fdcl::FFTS2_matrix_complex F = t.forward_transform(std::function<cd(double, double)>(f));
        cd* o = reinterpret_cast<cd*>(out);
        for (int l = 0; l <= L; ++l)
            for (int m = -l; m <= l; ++m) o[s2_idx(l, m)] = F(l, m);
    });
}

// fdcl::FFTS2_real::forward_transform (fdcl_FFTS2.cpp:424-448): out = packed real F
int ref_s2_forward_real(int L, const double* grid, double* out)
{
    return guarded([&] {
        const int B = L + 1, N = 2 * B;
        fdcl::FFTS2_real t(L);
        auto f = [&](double th, double ph) -> double { return grid[(long)k_of(th, B) * N + j_of(ph, B)]; };
        fdcl::FFTS2_matrix_real F = t.forward_transform(std::function<double(double, double)>(f));
        for (int l = 0; l <= L; ++l)
            for (int m = -l; m <= l; ++m) out[s2_idx(l, m)] = F(l, m);
    });
}

// fdcl::FFTS2_complex::inverse_transform(F, theta, phi): out = (re, im)
int ref_s2_inverse_complex_point(int L, const double* coeffs, double th, double ph, double* out)
{
    return guarded([&] {
        fdcl::FFTS2_complex t(L);
        fdcl::FFTS2_matrix_complex F(L);
        s2_unpack(L, reinterpret_cast<const cd*>(coeffs), F);
        const cd v = t.inverse_transform(F, th, ph);
        out[0] = v.real();
        out[1] = v.imag();
    });
}

// fdcl::FFTS2_real::inverse_transform(F, theta, phi)
int ref_s2_inverse_real_point(int L, const double* coeffs, double th, double ph, double* out)
{
    return guarded([&] {
        fdcl::FFTS2_real t(L);
        fdcl::FFTS2_matrix_real F(L);
        s2_unpack(L, coeffs, F);
        out[0] = t.inverse_transform(F, th, ph);
    });
}

// fdcl::Clebsch_Gordon_complex::compute(l1, l2) (fdcl_Clebsch_Gordon.cpp): the coefficient matrix C,
// ((2 l1 + 1)(2 l2 + 1))^2 entries, column-major; *dim receives its order
int ref_clebsch_gordan_complex(int l1, int l2, double* out, int* dim)
{
    return guarded([&] {
        fdcl::Clebsch_Gordon_complex c(l1, l2);
        c.compute(l1, l2);
        *dim = c.C.rows();
        if (out)
            for (int j = 0; j < c.C.cols(); ++j)
                for (int i = 0; i < c.C.rows(); ++i) out[(long)j * c.C.rows() + i] = c.C(i, j);
    });
}

}  // extern "C"
