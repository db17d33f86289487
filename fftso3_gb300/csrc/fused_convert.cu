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
// The group-major place of (l, m, n) and its inverse are closed-form (no table lookups), each CTA serves one
// bucket, and the gathers stay inside one function's coefficients (a few MB at l_max = 64), which the
// neighbouring threads of the launch read at the same time, so they are served by L2.
#include "common.cuh"
#include "fused.cuh"
#include "rsph.cuh"

namespace fftso3 {

namespace {

// The group-major layout in closed form (the order the tensor-core plans build their offsets in, group by group
// g = m0^2 + m0 + n0, pairs of group_pairs(), rows l = m0..L): the groups of one m0 >= 1 hold 8 m0 runs of
// B - m0 rows -- n0 = -m0 (2 pairs), -m0 < n0 < m0 (4 pairs each), n0 = m0 (2 pairs) -- after the single run
// of m0 = 0.
__device__ __forceinline__ int block_start(int m0, int B)  // < 2^31 for B <= 256
{
    if (m0 == 0) return 0;
    const int ab = (m0 - 1) * m0;
    return B + 8 * (B * (ab / 2) - ab * (2 * m0 - 1) / 6);
}

__device__ __forceinline__ int run_index(int m0, int n0, int pp)
{
    if (m0 == 0) return 0;
    if (n0 == -m0) return pp;
    if (n0 == m0) return 8 * m0 - 2 + pp;
    return 2 + 4 * (n0 + m0 - 1) + pp;
}

// group-major offset of F(l, m, n) in a bucket of bandwidth B
__device__ __forceinline__ long long gm_offset(int l, int m, int n, int B)
{
    int g, pp;
    pair_of(m, n, g, pp);
    const int am = m < 0 ? -m : m, an = n < 0 ? -n : n, m0 = am > an ? am : an;
    const int n0 = g - m0 * m0 - m0;
    return block_start(m0, B) + (long long)run_index(m0, n0, pp) * (B - m0) + (l - m0);
}

// largest l with l (4 l^2 - 1) / 3 <= r (the packed offset of degree l; < 2^31 for l <= 256)
__device__ __forceinline__ int off32(int l) { return l * (4 * l * l - 1) / 3; }
__device__ __forceinline__ int degree_of(int r)
{
    int l = (int)cbrtf(0.75f * (float)r);
    while (l > 0 && off32(l) > r) --l;
    while (off32(l + 1) <= r) ++l;
    return l;
}


template <bool REAL>
__global__ void __launch_bounds__(CONVERT_THREADS) fused_group_to_packed_kernel(const BucketSeg* __restrict__ segs,
                                                                                const unsigned short* __restrict__ cseg,
                                                                                void* __restrict__ out)
{
    const BucketSeg& S = segs[cseg[blockIdx.x]];
    const int B = S.B;
    const int C = (int)so3_off(B);
    const long long u = (blockIdx.x - S.cblk0) * (long long)CONVERT_THREADS + threadIdx.x;
    if (u >= (long long)S.batch * C) return;
    const int f = (int)(u / C), r = (int)(u - (long long)f * C);
    const int l = degree_of(r);
    const int W = 2 * l + 1, wi = r - off32(l);
    const int m = wi % W - l, n = wi / W - l;
    const float2* __restrict__ fg = S.fg + (long long)f * C;
    if (!REAL) {
        reinterpret_cast<float2*>(out)[S.c0 + u] = fg[gm_offset(l, m, n, B)];
        return;
    }
    const int am[2] = {-m, m}, bn[2] = {-n, n};
    const int na = (m == 0) ? 1 : 2, nb = (n == 0) ? 1 : 2;
    float2 v[2][2];
    for (int ia = 0; ia < na; ++ia)
        for (int ib = 0; ib < nb; ++ib) v[ia][ib] = fg[gm_offset(l, am[ia], bn[ib], B)];
    float acc = 0.f;
    for (int ia = 0; ia < na; ++ia)
        for (int ib = 0; ib < nb; ++ib) {
            const c2t<float> t1 = tmat_t<float>(m, am[ia]), t2 = conj_t(tmat_t<float>(n, bn[ib]));
            const c2t<float> c = cmul_t(cmul_t(t1, c2t<float>{v[ia][ib].x, v[ia][ib].y}), t2);
            acc += c.x;
        }
    reinterpret_cast<float*>(out)[S.c0 + u] = acc;
}

template <bool REAL>
__global__ void __launch_bounds__(CONVERT_THREADS) fused_packed_to_group_kernel(const BucketSeg* __restrict__ segs,
                                                                                const unsigned short* __restrict__ cseg,
                                                                                const void* __restrict__ in)
{
    const BucketSeg& S = segs[cseg[blockIdx.x]];
    const int B = S.B;
    const int C = (int)so3_off(B);
    const long long u = (blockIdx.x - S.cblk0) * (long long)CONVERT_THREADS + threadIdx.x;
    if (u >= (long long)S.batch * C) return;
    const int f = (int)(u / C), e = (int)(u - (long long)f * C);
    int lo = 0, hi = B - 1;  // m0: the block holding e
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (block_start(mid, B) <= e) lo = mid;
        else hi = mid - 1;
    }
    const int m0 = lo, nl = B - m0;
    const int rel = e - block_start(m0, B), ri = rel / nl, l = m0 + rel - ri * nl;
    int n0, pp;
    if (m0 == 0) { n0 = 0; pp = 0; }
    else if (ri < 2) { n0 = -m0; pp = ri; }
    else if (ri >= 8 * m0 - 2) { n0 = m0; pp = ri - (8 * m0 - 2); }
    else { n0 = -m0 + 1 + (ri - 2) / 4; pp = (ri - 2) & 3; }
    // pair pp of group_pairs(m0, n0), without its table (which a dynamic index would put in local memory)
    const int sgn = ((m0 + n0) & 1) ? -1 : 1;
    const int m = pp == 0 ? m0 : pp == 1 ? -m0 : pp == 2 ? n0 : -n0;
    const int n = pp == 0 ? n0 : pp == 1 ? -n0 : pp == 2 ? m0 : -m0;
    const int psign = (pp == 1 || pp == 2) ? sgn : 1;
    float2 v;
    if (!REAL) {
        v = reinterpret_cast<const float2*>(in)[S.c0 + (long long)f * C + so3_idx(l, m, n)];
    } else {
        const float* __restrict__ fr = reinterpret_cast<const float*>(in) + S.c0 + (long long)f * C;
        const int am[2] = {m, -m}, bn[2] = {n, -n};
        const int na = (m == 0) ? 1 : 2, nb = (n == 0) ? 1 : 2;
        float x[2][2];
        for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) x[ia][ib] = fr[so3_idx(l, am[ia], bn[ib])];
        c2t<float> acc = {0.f, 0.f};
        for (int ia = 0; ia < na; ++ia)
            for (int ib = 0; ib < nb; ++ib) {
                const c2t<float> c = cmul_t(conj_t(tmat_t<float>(am[ia], m)), tmat_t<float>(bn[ib], n));
                acc.x += c.x * x[ia][ib];
                acc.y += c.y * x[ia][ib];
            }
        v = make_float2(acc.x, acc.y);
    }
    const float sc = (float)(2 * l + 1) * (float)psign;
    S.fg[(long long)f * C + e] = make_float2(sc * v.x, sc * v.y);
}

}  // namespace

cudaError_t launch_fused_group_to_packed(const BucketSeg* segs, const unsigned short* cseg, long long nblk,
                                         bool real, void* out, cudaStream_t st)
{
    if (nblk <= 0) return cudaSuccess;
    if (nblk > 0x7fffffffLL) return cudaErrorInvalidValue;
    if (real)
        fused_group_to_packed_kernel<true><<<(unsigned)nblk, CONVERT_THREADS, 0, st>>>(segs, cseg, out);
    else
        fused_group_to_packed_kernel<false><<<(unsigned)nblk, CONVERT_THREADS, 0, st>>>(segs, cseg, out);
    return cudaGetLastError();
}

cudaError_t launch_fused_packed_to_group(const BucketSeg* segs, const unsigned short* cseg, long long nblk,
                                         bool real, const void* in, cudaStream_t st)
{
    if (nblk <= 0) return cudaSuccess;
    if (nblk > 0x7fffffffLL) return cudaErrorInvalidValue;
    if (real)
        fused_packed_to_group_kernel<true><<<(unsigned)nblk, CONVERT_THREADS, 0, st>>>(segs, cseg, in);
    else
        fused_packed_to_group_kernel<false><<<(unsigned)nblk, CONVERT_THREADS, 0, st>>>(segs, cseg, in);
    return cudaGetLastError();
}

}  // namespace fftso3
