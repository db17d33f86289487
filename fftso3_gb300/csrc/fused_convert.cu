// Coefficient conversions of an uneven SO(3) batch, every bucket in one launch (fused.cuh).
//
// The per-bucket plans convert in two launches each (contract_tc.cu: the tiled group-major <-> packed
// permutations, then the real-basis change so3_c2r / so3_r2c of contract_fp64.cu, fdcl_FFTSO3.cpp:1107-1139
// for matrix2rsph); here one thread forms one output coefficient of any bucket from the entries it needs,
// with the same arithmetic in the same order, so the results are the bucket plans' bit for bit:
//   forward: packed F(l, m, n) from the group-major GEMM output (real kinds: Re(T F T^H), the four
//            entries (l, +-m, +-n));
//   inverse: group-major (2l + 1) sign F(l, m, n) of the pair at that place (real kinds: F = T^H F_r T from
//            the four real entries (l, +-m, +-n)).
// The gathers are scattered but stay inside one function's coefficients (a few MB at l_max = 64), which the
// neighbouring threads of the launch read at the same time, so they are served by L2.
#include "common.cuh"
#include "fused.cuh"
#include "rsph.cuh"

namespace fftso3 {

namespace {

__device__ __forceinline__ int seg_of(const BucketSeg* __restrict__ segs, int nseg, long long t)
{
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (segs[mid].coef0 <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// largest l with so3_off(l) <= r
__device__ __forceinline__ int degree_of(long long r)
{
    int l = (int)cbrtf(0.75f * (float)r);
    while (l > 0 && so3_off(l) > r) --l;
    while (so3_off(l + 1) <= r) ++l;
    return l;
}

template <bool REAL>
__global__ void __launch_bounds__(256) fused_group_to_packed_kernel(const BucketSeg* __restrict__ segs, int nseg,
                                                                    long long ncoef, void* __restrict__ out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncoef) return;
    const BucketSeg& S = segs[seg_of(segs, nseg, t)];
    const int B = S.B;
    const long long C = so3_off(B), u = t - S.coef0, f = u / C, r = u - f * C;
    const int l = degree_of(r);
    const int W = 2 * l + 1, wi = (int)(r - so3_off(l));
    const int m = wi % W - l, n = wi / W - l;
    const float2* __restrict__ fg = S.fg + f * C;
    const long long* __restrict__ goff2 = S.goff2;
    auto val = [&](int mm, int nn) -> float2 {
        int g, pp;
        pair_of(mm, nn, g, pp);
        const int am = mm < 0 ? -mm : mm, an = nn < 0 ? -nn : nn, m0 = am > an ? am : an;
        return fg[goff2[g] + (long long)pp * (B - m0) + (l - m0)];
    };
    if (!REAL) {
        reinterpret_cast<float2*>(out)[S.c0 + u] = val(m, n);
        return;
    }
    const int am[2] = {-m, m}, bn[2] = {-n, n};
    const int na = (m == 0) ? 1 : 2, nb = (n == 0) ? 1 : 2;
    float acc = 0.f;
    for (int ia = 0; ia < na; ++ia)
        for (int ib = 0; ib < nb; ++ib) {
            const c2t<float> t1 = tmat_t<float>(m, am[ia]), t2 = conj_t(tmat_t<float>(n, bn[ib]));
            const float2 v = val(am[ia], bn[ib]);
            const c2t<float> c = cmul_t(cmul_t(t1, c2t<float>{v.x, v.y}), t2);
            acc += c.x;
        }
    reinterpret_cast<float*>(out)[S.c0 + u] = acc;
}

template <bool REAL>
__global__ void __launch_bounds__(256) fused_packed_to_group_kernel(const BucketSeg* __restrict__ segs, int nseg,
                                                                    long long ncoef, const void* __restrict__ in)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncoef) return;
    const BucketSeg& S = segs[seg_of(segs, nseg, t)];
    const int B = S.B;
    const long long C = so3_off(B), u = t - S.coef0, f = u / C, e = u - f * C;
    const long long* __restrict__ go = S.goff2;
    int lo = 0, hi = B * B - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (go[mid] <= e) lo = mid;
        else hi = mid - 1;
    }
    int m0, n0;
    group_mn(lo, m0, n0);
    const int nl = B - m0;
    const int off = (int)(e - go[lo]), pp = off / nl, l = m0 + off - pp * nl;
    const GroupPairs P = group_pairs(m0, n0);
    const int m = P.m[pp], n = P.n[pp];
    float2 v;
    if (!REAL) {
        v = reinterpret_cast<const float2*>(in)[S.c0 + f * C + so3_idx(l, m, n)];
    } else {
        const float* __restrict__ fr = reinterpret_cast<const float*>(in) + S.c0 + f * C;
        const int am[2] = {m, -m}, bn[2] = {n, -n};
        const int na = (m == 0) ? 1 : 2, nb = (n == 0) ? 1 : 2;
        c2t<float> acc = {0.f, 0.f};
        for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
                const c2t<float> c = cmul_t(conj_t(tmat_t<float>(am[ia], m)), tmat_t<float>(bn[ib], n));
                const float x = fr[so3_idx(l, am[ia], bn[ib])];
                acc.x += c.x * x;
                acc.y += c.y * x;
            }
        v = make_float2(acc.x, acc.y);
    }
    const float sc = (float)(2 * l + 1) * (float)P.sign[pp];
    S.fg[f * C + e] = make_float2(sc * v.x, sc * v.y);
}

unsigned blocks_of(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

cudaError_t launch_fused_group_to_packed(const BucketSeg* segs, int nseg, long long ncoef, bool real, void* out,
                                         cudaStream_t st)
{
    if (ncoef <= 0) return cudaSuccess;
    if ((ncoef + 255) / 256 > 0x7fffffffLL || nseg <= 0) return cudaErrorInvalidValue;
    if (real)
        fused_group_to_packed_kernel<true><<<blocks_of(ncoef), 256, 0, st>>>(segs, nseg, ncoef, out);
    else
        fused_group_to_packed_kernel<false><<<blocks_of(ncoef), 256, 0, st>>>(segs, nseg, ncoef, out);
    return cudaGetLastError();
}

cudaError_t launch_fused_packed_to_group(const BucketSeg* segs, int nseg, long long ncoef, bool real, const void* in,
                                         cudaStream_t st)
{
    if (ncoef <= 0) return cudaSuccess;
    if ((ncoef + 255) / 256 > 0x7fffffffLL || nseg <= 0) return cudaErrorInvalidValue;
    if (real)
        fused_packed_to_group_kernel<true><<<blocks_of(ncoef), 256, 0, st>>>(segs, nseg, ncoef, in);
    else
        fused_packed_to_group_kernel<false><<<blocks_of(ncoef), 256, 0, st>>>(segs, nseg, ncoef, in);
    return cudaGetLastError();
}

}  // namespace fftso3
