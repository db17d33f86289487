// C++ drop-in check: the reference's gtest cases for the transform classes
// (test/test.cpp:39-88, ASSERT_NEAR(err, 0, 1e-10) at l_max = 5) and README
// example0 (tr R -> F^1 = I/3, f(I) = 3), written against include/fdcl_gb300.hpp.
#include <cstdio>
#include <cmath>
#include "fdcl_gb300.hpp"

static int failures = 0;
static void expect_near(const char* what, double v, double ref, double tol)
{
    bool ok = std::fabs(v - ref) <= tol;
    std::printf("%-36s %.3e %s\n", what, v, ok ? "ok" : "FAIL");
    if (!ok) ++failures;
}

int main()
{
    const int l_max = 5;
    fdcl::FFTSO3_complex FFTSO3(l_max);
    fdcl::FFTSO3_real RFFTSO3(l_max);
    fdcl::FFTS2_complex FFTS2(l_max);
    fdcl::FFTS2_real RFFTS2(l_max);
    expect_near("FFTSO3Test.ComplexTransform", FFTSO3.check_transform(), 0., 1e-10);
    expect_near("FFTSO3Test.RealTransform", RFFTSO3.check_transform(), 0., 1e-10);
    expect_near("FFTS2Test.ComplexTransform", FFTS2.check_transform(), 0., 1e-10);
    expect_near("FFTS2Test.RealTransform", RFFTS2.check_transform(), 0., 1e-10);

    // README example0
    fdcl::FFTSO3_real R2(2);
    fdcl::FFTSO3_matrix_real F = R2.forward_transform([](fdcl::gb300::Mat3 R) { return R.trace(); });
    double err = 0.;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) err = std::fmax(err, std::fabs(F(1, i - 1, j - 1) - (i == j ? 1. / 3. : 0.)));
    expect_near("example0 F^1 = I/3", err, 0., 1e-14);
    fdcl::gb300::Mat3 I;
    expect_near("example0 f(I) = 3", R2.inverse_transform(F, I), 3., 1e-12);

    // point inverse agrees with the grid synthesis path (complex)
    fdcl::FFTSO3_matrix_complex G(4);
    G.setRandom();
    fdcl::FFTSO3_complex C4(4);
    std::complex<double> v = C4.inverse_transform(G, 0.3, 1.1, -0.4);
    std::complex<double> w = 0.;
    fdcl::FFTSO3_matrix_real d = C4.wigner_d(1.1);
    for (int l = 0; l <= 4; ++l)
        for (int m = -l; m <= l; ++m)
            for (int n = -l; n <= l; ++n)
                w += (double)(2 * l + 1) * G(l, m, n) * d(l, m, n) * std::exp(std::complex<double>(0, -m * 0.3 - n * (-0.4)));
    expect_near("point inverse vs direct sum", std::abs(v - w), 0., 1e-12);
    std::printf("%s\n", failures ? "FAILED" : "PASSED");
    return failures ? 1 : 0;
}
