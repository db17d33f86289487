// fdcl_gb300.hpp -- header-only C++ drop-in for the transform classes of
// fdcl-gwu/FFTSO3, running on the GB300 library through its C ABI
// (fftso3_gb300.h).
//
// Same names, signatures and argument meaning as the reference:
//   fdcl::FFTSO3_matrix<T>  (include/fdcl_FFTSO3_matrix.hpp:44-91): F(l,m,n), F[l], init, setZero,
//                            setRandom, norm, real, + - *, <<
//   fdcl::FFTS2_matrix<T>   (include/fdcl_FFTS2_matrix.hpp:40-86):  F(l,m), F[l], ...
//   fdcl::FFTSO3_complex / FFTSO3_real (include/fdcl_FFTSO3.hpp:27-308): init, forward_transform(func),
//                            forward_transform(func(R)), inverse_transform(F, a, b, g),
//                            inverse_transform(F, R), wigner_d(beta), check_transform()
//   fdcl::FFTS2_complex / FFTS2_real (include/fdcl_FFTS2.hpp:28-160)
// The per-l blocks are column-major (2l+1)x(2l+1) matrices (Eigen::MatrixXcd /
// MatrixXd when FFTSO3_GB300_WITH_EIGEN is defined, otherwise the small
// fdcl::gb300::Block type below, which offers the subset the reference's
// users touch: operator()(i,j), rows(), cols(), data(), norm(), setZero(),
// setRandom()).  Rotation arguments are Eigen::Matrix3d or fdcl::gb300::Mat3.
//
// The callback of forward_transform is sampled on the host (in parallel with
// OpenMP when enabled, as the reference calls it from OpenMP threads,
// fdcl_FFTSO3.cpp:675-685) and the transform runs on the GPU.  Errors throw
// std::runtime_error with the library's message (the reference asserts).
#ifndef FDCL_GB300_HPP
#define FDCL_GB300_HPP

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "fftso3_gb300.h"

#ifdef FFTSO3_GB300_WITH_EIGEN
#include <Eigen/Dense>
#endif

namespace fdcl {

using std::complex;

namespace gb300 {

inline void check(int rc)
{
    if (rc != FFTSO3_SUCCESS) throw std::runtime_error(std::string("fftso3: ") + fftso3_last_error_string());
}

#ifdef FFTSO3_GB300_WITH_EIGEN
template <class T> using Block = Eigen::Matrix<T, Eigen::Dynamic, Eigen::Dynamic>;
template <class T> using Vec = Eigen::Matrix<T, Eigen::Dynamic, 1>;
using Mat3 = Eigen::Matrix3d;
inline double mat3(const Mat3& R, int i, int j) { return R(i, j); }
#else
// Column-major dense block (the subset of Eigen::Matrix the containers expose).
template <class T> class Block {
public:
    Block() {}
    Block(int r, int c) { resize(r, c); }
    void resize(int r, int c)
    {
        r_ = r;
        c_ = c;
        d_.assign((size_t)r * c, T(0));
    }
    int rows() const { return r_; }
    int cols() const { return c_; }
    T& operator()(int i, int j) { return d_[(size_t)j * r_ + i]; }
    const T& operator()(int i, int j) const { return d_[(size_t)j * r_ + i]; }
    T& operator()(int i) { return d_[i]; }
    const T& operator()(int i) const { return d_[i]; }
    T* data() { return d_.data(); }
    const T* data() const { return d_.data(); }
    void setZero() { std::fill(d_.begin(), d_.end(), T(0)); }
    void setRandom() { for (auto& x : d_) x = rnd(x); }
    double norm() const
    {
        double s = 0.;
        for (const auto& x : d_) s += std::norm(complex<double>(x));
        return std::sqrt(s);
    }
    Block operator+(const Block& o) const { Block z = *this; for (size_t i = 0; i < d_.size(); ++i) z.d_[i] += o.d_[i]; return z; }
    Block operator-(const Block& o) const { Block z = *this; for (size_t i = 0; i < d_.size(); ++i) z.d_[i] -= o.d_[i]; return z; }
    template <class S> Block operator*(const S& s) const { Block z = *this; for (auto& x : z.d_) x *= s; return z; }

private:
    static double rnd(double) { return 2.0 * std::rand() / RAND_MAX - 1.0; }
    static complex<double> rnd(complex<double>)
    {
        double a = 2.0 * std::rand() / RAND_MAX - 1.0, b = 2.0 * std::rand() / RAND_MAX - 1.0;
        return {a, b};
    }
    int r_ = 0, c_ = 0;
    std::vector<T> d_;
};
template <class T> using Vec = Block<T>;
struct Mat3 {
    double a[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};  // column-major
    double& operator()(int i, int j) { return a[j * 3 + i]; }
    double operator()(int i, int j) const { return a[j * 3 + i]; }
    double trace() const { return a[0] + a[4] + a[8]; }
    void setIdentity() { *this = Mat3(); }
};
inline double mat3(const Mat3& R, int i, int j) { return R(i, j); }
#endif

// misc_matrix_func.cpp:144-177 (R2Euler323, Euler3232R)
inline void R2Euler323(const Mat3& R, double& a, double& b, double& g)
{
    b = std::acos(std::fmax(-1.0, std::fmin(1.0, mat3(R, 2, 2))));
    if (b != 0.) {
        g = std::atan2(mat3(R, 2, 1), -mat3(R, 2, 0));
        a = std::atan2(mat3(R, 1, 2), mat3(R, 0, 2));
    } else {
        a = std::acos(std::fmax(-1.0, std::fmin(1.0, mat3(R, 0, 0)))) / 2.;
        g = a;
    }
}

inline Mat3 Euler3232R(double a, double b, double g)
{
    Mat3 R;
    const double ca = std::cos(a), sa = std::sin(a), cb = std::cos(b), sb = std::sin(b), cg = std::cos(g),
                 sg = std::sin(g);
    R(0, 0) = ca * cb * cg - sa * sg;  R(0, 1) = -cg * sa - ca * cb * sg;  R(0, 2) = ca * sb;
    R(1, 0) = ca * sg + cb * cg * sa;  R(1, 1) = ca * cg - cb * sa * sg;   R(1, 2) = sa * sb;
    R(2, 0) = -cg * sb;                R(2, 1) = sb * sg;                  R(2, 2) = cb;
    return R;
}

// Owns one plan (created lazily for the current l_max).
class PlanHolder {
public:
    ~PlanHolder() { reset(); }
    void reset()
    {
        if (p_) fftso3_plan_destroy(p_);
        p_ = nullptr;
    }
    fftso3_plan* get(int kind, int l_max)
    {
        if (!p_ || kind != kind_ || l_max != l_max_) {
            reset();
            check(fftso3_plan_create(&p_, kind, l_max, 1, FFTSO3_PREC_FP64, recursion, 0));
            kind_ = kind;
            l_max_ = l_max;
        }
        return p_;
    }
    int recursion = FFTSO3_RECURSION_REFERENCE;

private:
    fftso3_plan* p_ = nullptr;
    int kind_ = -1, l_max_ = -1;
};

inline double beta_k(int B, int k) { return ((double)(2 * k + 1)) * M_PI / 4. / ((double)B); }
inline double alpha_j(int B, int j) { return ((double)j) * M_PI / ((double)B); }

}  // namespace gb300

// ---------------------------------------------------------------- containers

template <class ScalarType> class FFTSO3_matrix {
public:
    int l_max = 0;
    std::vector<gb300::Block<ScalarType>> M;
    FFTSO3_matrix() {}
    explicit FFTSO3_matrix(int l) { init(l); }
    void init(int l)
    {
        l_max = l;
        M.resize(l + 1);
        for (int i = 0; i <= l; ++i) {
            M[i].resize(2 * i + 1, 2 * i + 1);
            M[i].setZero();
        }
    }
    gb300::Block<ScalarType>& operator[](int l) { chk(l); return M[l]; }
    ScalarType& operator()(int l, int m, int n)
    {
        chk(l);
        if (std::min(m, n) < -l || std::max(m, n) > l) throw std::out_of_range("FFTSO3_matrix index");
        return M[l](m + l, n + l);
    }
    void setRandom() { for (auto& b : M) b.setRandom(); }
    void setZero() { for (auto& b : M) b.setZero(); }
    double norm() const
    {
        double y = 0.;
        for (const auto& b : M) y += b.norm();
        return y;
    }
    FFTSO3_matrix<double> real() const
    {
        FFTSO3_matrix<double> Z(l_max);
        for (int l = 0; l <= l_max; ++l)
            for (int j = 0; j < 2 * l + 1; ++j)
                for (int i = 0; i < 2 * l + 1; ++i) Z.M[l](i, j) = std::real(complex<double>(M[l](i, j)));
        return Z;
    }
    FFTSO3_matrix operator+(const FFTSO3_matrix& o) const { FFTSO3_matrix z(l_max); for (int l = 0; l <= l_max; ++l) z.M[l] = M[l] + o.M[l]; return z; }
    FFTSO3_matrix operator-(const FFTSO3_matrix& o) const { FFTSO3_matrix z(l_max); for (int l = 0; l <= l_max; ++l) z.M[l] = M[l] - o.M[l]; return z; }
    FFTSO3_matrix operator*(const double& c) const { FFTSO3_matrix z(l_max); for (int l = 0; l <= l_max; ++l) z.M[l] = M[l] * c; return z; }
    // packed copy: the per-l column-major blocks end to end (the C ABI layout)
    void pack(ScalarType* out) const
    {
        size_t o = 0;
        for (const auto& b : M) {
            std::memcpy(out + o, b.data(), sizeof(ScalarType) * b.rows() * b.cols());
            o += (size_t)b.rows() * b.cols();
        }
    }
    void unpack(const ScalarType* in)
    {
        size_t o = 0;
        for (auto& b : M) {
            std::memcpy(b.data(), in + o, sizeof(ScalarType) * b.rows() * b.cols());
            o += (size_t)b.rows() * b.cols();
        }
    }
    size_t size() const { size_t n = 0; for (const auto& b : M) n += (size_t)b.rows() * b.cols(); return n; }

private:
    void chk(int l) const { if (l < 0 || l > l_max) throw std::out_of_range("FFTSO3_matrix degree"); }
};

template <class T> std::ostream& operator<<(std::ostream& os, const FFTSO3_matrix<T>& F)
{
    for (int l = 0; l <= F.l_max; ++l) {
        os << "l=" << l << "\n";
        for (int i = 0; i < 2 * l + 1; ++i) {
            for (int j = 0; j < 2 * l + 1; ++j) os << F.M[l](i, j) << " ";
            os << "\n";
        }
        os << "\n";
    }
    return os;
}

typedef FFTSO3_matrix<double> FFTSO3_matrix_real;
typedef FFTSO3_matrix<complex<double>> FFTSO3_matrix_complex;

template <class ScalarType> class FFTS2_matrix {
public:
    int l_max = 0;
    std::vector<gb300::Vec<ScalarType>> M;
    FFTS2_matrix() {}
    explicit FFTS2_matrix(int l) { init(l); }
    void init(int l)
    {
        l_max = l;
        M.resize(l + 1);
        for (int i = 0; i <= l; ++i) {
            M[i].resize(2 * i + 1, 1);
            M[i].setZero();
        }
    }
    gb300::Vec<ScalarType>& operator[](int l) { return M[l]; }
    ScalarType& operator()(int l, int m)
    {
        if (l < 0 || l > l_max || m < -l || m > l) throw std::out_of_range("FFTS2_matrix index");
        return M[l](m + l);
    }
    void setRandom() { for (auto& b : M) b.setRandom(); }
    void setZero() { for (auto& b : M) b.setZero(); }
    double norm() const { double y = 0.; for (const auto& b : M) y += b.norm(); return y; }
    FFTS2_matrix operator-(const FFTS2_matrix& o) const { FFTS2_matrix z(l_max); for (int l = 0; l <= l_max; ++l) z.M[l] = M[l] - o.M[l]; return z; }
    FFTS2_matrix operator+(const FFTS2_matrix& o) const { FFTS2_matrix z(l_max); for (int l = 0; l <= l_max; ++l) z.M[l] = M[l] + o.M[l]; return z; }
    void pack(ScalarType* out) const { size_t o = 0; for (const auto& b : M) { std::memcpy(out + o, b.data(), sizeof(ScalarType) * b.rows()); o += b.rows(); } }
    void unpack(const ScalarType* in) { size_t o = 0; for (auto& b : M) { std::memcpy(b.data(), in + o, sizeof(ScalarType) * b.rows()); o += b.rows(); } }
    size_t size() const { size_t n = 0; for (const auto& b : M) n += b.rows(); return n; }
};

typedef FFTS2_matrix<double> FFTS2_matrix_real;
typedef FFTS2_matrix<complex<double>> FFTS2_matrix_complex;

// ---------------------------------------------------------------- transforms

class FFTSO3_complex {
public:
    int l_max = 0;
    bool check_verbose = false;
    FFTSO3_complex() {}
    explicit FFTSO3_complex(int l) { init(l); }
    virtual ~FFTSO3_complex() {}
    void init(int l)
    {
        l_max = l;
        B = l + 1;
    }
    // FFTSO3_RECURSION_REFERENCE (default, bit-faithful) or FFTSO3_RECURSION_STABLE
    void set_recursion(int r) { plan_.recursion = r; plan_.reset(); }

    FFTSO3_matrix_complex forward_transform(std::function<complex<double>(double, double, double)> func)
    {
        const int N = 2 * B;
        std::vector<complex<double>> grid((size_t)N * N * N);
#pragma omp parallel for collapse(2)
        for (int k = 0; k < N; ++k)
            for (int j1 = 0; j1 < N; ++j1)
                for (int j2 = 0; j2 < N; ++j2)
                    grid[((size_t)k * N + j1) * N + j2] =
                        func(gb300::alpha_j(B, j1), gb300::beta_k(B, k), gb300::alpha_j(B, j2));
        FFTSO3_matrix_complex F(l_max);
        std::vector<complex<double>> c(F.size());
        gb300::check(fftso3_forward_host(plan_.get(FFTSO3_SO3_COMPLEX, l_max), grid.data(), c.data(), nullptr));
        F.unpack(c.data());
        return F;
    }
    FFTSO3_matrix_complex forward_transform(std::function<complex<double>(gb300::Mat3)> func)
    {
        return forward_transform([=](double a, double b, double g) { return func(gb300::Euler3232R(a, b, g)); });
    }
    complex<double> inverse_transform(FFTSO3_matrix_complex F, double alpha, double beta, double gamma)
    {
        init(F.l_max);  // as the reference (fdcl_FFTSO3.cpp:500)
        return point(F, alpha, beta, gamma);
    }
    complex<double> inverse_transform(FFTSO3_matrix_complex F, gb300::Mat3 R)
    {
        double a, b, g;
        gb300::R2Euler323(R, a, b, g);
        return inverse_transform(F, a, b, g);
    }
    FFTSO3_matrix_real wigner_d(double beta)
    {
        FFTSO3_matrix_real d(l_max);
        std::vector<double> buf(d.size());
        gb300::check(fftso3_wigner_d(beta, l_max, plan_.recursion, buf.data()));
        d.unpack(buf.data());
        return d;
    }
    // fdcl_FFTSO3.cpp:598-610
    double check_transform()
    {
        F_4_check.init(l_max);
        F_4_check.setRandom();
        FFTSO3_matrix_complex G = grid_roundtrip(F_4_check);
        return (F_4_check - G).norm();
    }

protected:
    int B = 1;
    gb300::PlanHolder plan_;
    FFTSO3_matrix_complex F_4_check;

    complex<double> point(FFTSO3_matrix_complex& F, double a, double b, double g)
    {
        // coefficients on the device for the point kernel: go through the host-buffer inverse path
        fftso3_plan* p = plan_.get(FFTSO3_SO3_COMPLEX, l_max);
        std::vector<complex<double>> c(F.size());
        F.pack(c.data());
        void* d = nullptr;
        if (cudaMalloc(&d, sizeof(complex<double>) * c.size()) != cudaSuccess)
            throw std::runtime_error("device allocation failed");
        cudaMemcpy(d, c.data(), sizeof(complex<double>) * c.size(), cudaMemcpyHostToDevice);
        double pts[3] = {a, b, g};
        complex<double> out;
        int rc = fftso3_inverse_points(p, d, 0, pts, 1, &out, nullptr);
        cudaFree(d);
        gb300::check(rc);
        return out;
    }
    FFTSO3_matrix_complex grid_roundtrip(FFTSO3_matrix_complex& F)
    {
        const int N = 2 * B;
        fftso3_plan* p = plan_.get(FFTSO3_SO3_COMPLEX, l_max);
        std::vector<complex<double>> c(F.size()), g((size_t)N * N * N), c2(F.size());
        F.pack(c.data());
        gb300::check(fftso3_inverse_host(p, c.data(), g.data(), nullptr));
        gb300::check(fftso3_forward_host(p, g.data(), c2.data(), nullptr));
        FFTSO3_matrix_complex G(l_max);
        G.unpack(c2.data());
        return G;
    }
};

class FFTSO3_real : public FFTSO3_complex {
public:
    FFTSO3_real() {}
    explicit FFTSO3_real(int l) { init(l); }
    FFTSO3_matrix_real forward_transform(std::function<double(double, double, double)> func)
    {
        const int N = 2 * B;
        std::vector<double> grid((size_t)N * N * N);
#pragma omp parallel for collapse(2)
        for (int k = 0; k < N; ++k)
            for (int j1 = 0; j1 < N; ++j1)
                for (int j2 = 0; j2 < N; ++j2)
                    grid[((size_t)k * N + j1) * N + j2] =
                        func(gb300::alpha_j(B, j1), gb300::beta_k(B, k), gb300::alpha_j(B, j2));
        FFTSO3_matrix_real F(l_max);
        std::vector<double> c(F.size());
        gb300::check(fftso3_forward_host(plan_.get(FFTSO3_SO3_REAL, l_max), grid.data(), c.data(), nullptr));
        F.unpack(c.data());
        return F;
    }
    FFTSO3_matrix_real forward_transform(std::function<double(gb300::Mat3)> func)
    {
        return forward_transform([=](double a, double b, double g) { return func(gb300::Euler3232R(a, b, g)); });
    }
    double inverse_transform(FFTSO3_matrix_real F, double alpha, double beta, double gamma)
    {
        init(F.l_max);
        fftso3_plan* p = plan_.get(FFTSO3_SO3_REAL, l_max);
        std::vector<double> c(F.size());
        F.pack(c.data());
        void* d = nullptr;
        if (cudaMalloc(&d, sizeof(double) * c.size()) != cudaSuccess)
            throw std::runtime_error("device allocation failed");
        cudaMemcpy(d, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice);
        double pts[3] = {alpha, beta, gamma};
        double out = 0.;
        int rc = fftso3_inverse_points(p, d, 0, pts, 1, &out, nullptr);
        cudaFree(d);
        gb300::check(rc);
        return out;
    }
    double inverse_transform(FFTSO3_matrix_real F, gb300::Mat3 R)
    {
        double a, b, g;
        gb300::R2Euler323(R, a, b, g);
        return inverse_transform(F, a, b, g);
    }
    // fdcl_FFTSO3.cpp:1785-1797
    double check_transform()
    {
        FFTSO3_matrix_real F(l_max);
        F.setRandom();
        const int N = 2 * B;
        fftso3_plan* p = plan_.get(FFTSO3_SO3_REAL, l_max);
        std::vector<double> c(F.size()), g((size_t)N * N * N), c2(F.size());
        F.pack(c.data());
        gb300::check(fftso3_inverse_host(p, c.data(), g.data(), nullptr));
        gb300::check(fftso3_forward_host(p, g.data(), c2.data(), nullptr));
        FFTSO3_matrix_real G(l_max);
        G.unpack(c2.data());
        return (F - G).norm();
    }
};

template <class S, int KIND>
class FFTS2_base {
public:
    int l_max = 0;
    bool check_verbose = false;
    FFTS2_base() {}
    explicit FFTS2_base(int l) { init(l); }
    void init(int l)
    {
        l_max = l;
        B = l + 1;
    }
    FFTS2_matrix<S> forward_transform(std::function<S(double, double)> func)
    {
        const int N = 2 * B;
        std::vector<S> grid((size_t)N * N);
#pragma omp parallel for
        for (int k = 0; k < N; ++k)
            for (int j = 0; j < N; ++j) grid[(size_t)k * N + j] = func(gb300::beta_k(B, k), gb300::alpha_j(B, j));
        FFTS2_matrix<S> F(l_max);
        std::vector<S> c(F.size());
        gb300::check(fftso3_forward_host(plan_.get(KIND, l_max), grid.data(), c.data(), nullptr));
        F.unpack(c.data());
        return F;
    }
    // fdcl_FFTS2.cpp:302-316 / :481-493
    double check_transform()
    {
        FFTS2_matrix<S> F(l_max);
        F.setRandom();
        const int N = 2 * B;
        fftso3_plan* p = plan_.get(KIND, l_max);
        std::vector<S> c(F.size()), g((size_t)N * N), c2(F.size());
        F.pack(c.data());
        gb300::check(fftso3_inverse_host(p, c.data(), g.data(), nullptr));
        gb300::check(fftso3_forward_host(p, g.data(), c2.data(), nullptr));
        FFTS2_matrix<S> G(l_max);
        G.unpack(c2.data());
        return (F - G).norm();
    }

protected:
    int B = 1;
    gb300::PlanHolder plan_;
};

class FFTS2_complex : public FFTS2_base<complex<double>, FFTSO3_S2_COMPLEX> {
public:
    using FFTS2_base::FFTS2_base;
};
class FFTS2_real : public FFTS2_base<double, FFTSO3_S2_REAL> {
public:
    using FFTS2_base::FFTS2_base;
};

}  // namespace fdcl

#endif  // FDCL_GB300_HPP
