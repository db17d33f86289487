// Exact tensor-core inverse for the residual refinement of the SO(3) FP32-data
// transforms (FFTSO3_FLAG_REFINE), sm_103a.
//
// The refinement F += forward(f - inverse(F)) removes the first forward's error
// only if inverse(F) is formed far more accurately than the FP32 path's ~3e-7
// (the residual is ~5e-7 of f).  Its contraction
//   H_k(m, n) = sum_l (2l+1) F(l, m, n) d^l_mn(beta_k)        (fdcl_FFTSO3.cpp:498-531, on the grid)
// costs 8BC flops per function, which the FP64 units of this part run at ~1.2
// TFLOP/s.  This file runs it on the BF16 tensor cores with exact accumulation
// (the Ozaki splitting of a product into digit products):
//
//  * both operands are written as 2^E sum_{i<4} s_i 2^{-7-8i} with integer
//    digits |s_i| <= 128 (exact in BF16): the table T_g[l][k] = d^l(beta_k) with
//    one exponent per (group, k), the coefficients Y_g[l][c] = (2l+1) sign F(l, pair)
//    (formed exactly, as a double-float product) with one per (function, group,
//    pair) -- along the contracted degree l every digit of a column shares one
//    unit.  The factor (2l+1) sits on the coefficient side because the table's
//    values then keep a small range along l: a digit split is accurate to 2^-31 of
//    a column's largest value, and (2l+1) d ranges over ~9 more bits than d does;
//  * the digit products s_i t_j with i + j = v accumulate in FP32 TMEM
//    accumulator v (v = 0..3).  Every partial sum is an integer multiple of that
//    accumulator's unit below 2^24 (|s_i t_j| <= 2^14, at most 256 degrees -- the
//    reason for l_max <= 255 -- and at most 4 products per level), so the tensor
//    cores add them without rounding;
//  * the epilogue combines the four levels in double-float and scales by 2^E,
//    giving H to about 2^-30 of its largest term (the dropped products
//    i + j >= 4 and the digits below 2^-31), as double-float pencils.
// Grid form (N not a power of two from 64 to 512): a double-float FFT over
// (p, q) then gives the grid g, and the residual r = f - g is formed against
// the FP32 samples in the same arithmetic (f is exact there) and rounded to
// FP32 only as the small difference.  Spectral form (N = 64..512): the
// samples' FFT in double-float (pencils hi + lo), and the epilogue writes
// r^ = (hi + lo) - N^2 H at the forward pencil place of each (m, n) instead
// of H -- the FFT of the synthesised grid is N^2 H -- so neither g nor an
// FFT of the residual is formed.
//
// The coefficients' digits are formed once per chunk (digit_image_kernel) as the shared-memory image of each
// K step, so the kernel's B operand arrives by one bulk copy per stage.
// Kernel layout (one CTA per SM, persistent over (group, 128 k, 8 functions) items):
//   warp 0     TMA of the four table digit planes (MN-major operand, 128-byte swizzle) and bulk copy of the
//              coefficients' 32 KB digit-image tile;
//   warp 1     TMEM owner (512 columns: 2 buffers x 4 levels x 64) and MMA issuer:
//              A_j x [B_0 .. B_{3-j}] as one MMA of N = (4 - j) 64 into levels j..3,
//              so the 10 digit products take 4 instructions per 16 degrees;
//   warps 2-9  epilogue, two warps per TMEM lane quarter: TMEM -> double-float H -> pencils [fn][p][q][k]
//              (or the spectral residual).
// Every mbarrier wait is bounded (~1 s); on timeout the kernel records an error
// code in the state's error word and unwinds, freeing its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/fftso3_gb300.h"
#include "common.cuh"
#include "df32.cuh"
#include "fft.cuh"
#include "refine_oz.cuh"
#include "tc.cuh"
#include "tc_ptx.cuh"

namespace fftso3 {

namespace oz {

using namespace ptx;

constexpr int BM = 128;                 // k rows per tile (TMEM lanes)
constexpr int BN = 64;                  // columns: 8 functions x 4 pairs x re/im
constexpr int FPT = BN / 8;             // functions per column tile
constexpr int BK = 64;                  // degrees per stage (one 128-byte swizzle row of BF16)
constexpr int UK = 16;                  // K per tcgen05.mma (kind::f16)
constexpr int NS = 4;                   // digits per operand = accumulation levels
constexpr int STAGES = 2;
constexpr int APLANE = BM * BK * 2;     // 16 KB: 128 k x 64 l (two 64 x 64 boxes)
constexpr int BPLANE = BN * BK * 2;     // 8 KB: 64 columns x 64 l
constexpr int STAGE_A = NS * APLANE;
constexpr int STAGE_B = NS * BPLANE;    // 32 KB: one tile of the coefficients' digit image
constexpr int STAGE_BYTES = STAGE_A + STAGE_B;
constexpr int NEPI = 8;                 // epilogue warps: two per TMEM lane quarter, each half of the columns
constexpr int THREADS = 32 * (2 + NEPI);
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 256 /*barriers*/ + 1024 /*alignment*/;
constexpr int ACC = NS * BN;            // TMEM columns of one accumulator buffer (levels 0..3)
constexpr int TMEM_COLS = 2 * ACC;
constexpr int EXP_MIN = -120, EXP_MAX = 120;
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert(TMEM_COLS == 512, "TMEM");

struct Args {
    const int4* items;      // (group, row tile, column tile, m0 << 16 | (n0 + 32768))
    const int2* iaux;       // per item: (group-major offset goff2[g], first table row grow0[g])
    int nitems;
    int L, N, batch, ngroups;
    long long fstride;      // pencil elements per function (N^3)
    const unsigned char* bimg;  // the coefficients' digit image: [column tile][group tile gt0[g] + step] x STAGE_B
    const int* gt0;             // first tile of each group in the image
    long long nbt;              // tiles per column tile
    const signed char* ey;  // exponents [fn][group][pair]
    const signed char* et;  // exponents [group][k]
    float4* pout;           // double-float pencils [fn][p][q][k]
    // spectral residual (rhi non-null): instead of H, write r = (rhi + rlo) - N^2 H at the forward pencil place
    // (-m, -n) of each (m, n), into rhi (complex64 pencils [fn][p][q][k]; rlo the remainders); e2n = log2 N^2
    float2* rhi;
    const float2* rlo;
    int e2n;
    int* err;
};

__device__ __forceinline__ void item_mn(const int4& it, int& m0, int& n0)
{
    m0 = it.w >> 16;
    n0 = (it.w & 0xFFFF) - 32768;
}

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// 2^e as a float for e in [-126, 127] (exact)
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }

// Digits of x = (h + l) sc (|x| <= 1): x 2^7 = s0 + s1 2^-8 + s2 2^-16 + s3 2^-24 + rest,
// each |s_i| <= 128 an integer (exact in BF16); every step but the first is exact in FP32.
__device__ __forceinline__ void digits4(float h, float l, float sc, float (&s)[NS])
{
    const float t = (h * sc) * 128.f;
    s[0] = rintf(t);
    float r = (t - s[0]) + (l * sc) * 128.f;
#pragma unroll
    for (int i = 1; i < NS; ++i) {
        r *= 256.f;
        s[i] = rintf(r);
        r -= s[i];
    }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);  // .x = a (low half)
    return *reinterpret_cast<const uint32_t*>(&v);
}

// level sums a_v (integers in units 2^-8v of level 0) -> double-float a_0 + 2^-8 a_1 + 2^-16 a_2 + 2^-24 a_3
__device__ __forceinline__ df32 combine_levels(float a0, float a1, float a2, float a3)
{
    const df32 s = df_two_sum(a0, a1 * 0.00390625f);
    return df_quick_two_sum(s.h, s.l + (a2 * 1.52587890625e-05f + a3 * 5.9604644775390625e-08f));
}

__global__ void __launch_bounds__(THREADS, 1)
    oz_inv_kernel(const __grid_constant__ CUtensorMap t0, const __grid_constant__ CUtensorMap t1,
                  const __grid_constant__ CUtensorMap t2, const __grid_constant__ CUtensorMap t3,
                  const __grid_constant__ Args a)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;
    uint64_t* acce = accf + 2;
    uint32_t* tmem_slot = (uint32_t*)(acce + 2);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto nsteps = [&](const int4& it) {
        int m0, n0;
        item_mn(it, m0, n0);
        return (a.L + 1 - m0 + BK - 1) / BK;
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], NEPI);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- TMA producer: the table digit planes and the coefficients' digit image
            const CUtensorMap* tm[NS] = {&t0, &t1, &t2, &t3};
            int kc = 0;
            for (int it = blockIdx.x; it < a.nitems && !*abort_flag; it += gridDim.x) {
                const int4 item = a.items[it];
                const int row0 = a.iaux[it].y;
                const int nk = nsteps(item);
                for (int i = 0; i < nk; ++i, ++kc) {
                    const int s = kc % STAGES;
                    if (kc >= STAGES && !mbar_wait(&empty[s], ((kc / STAGES) - 1) & 1, a.err, 21)) {
                        *abort_flag = 1;
                        break;
                    }
                    unsigned char* st = smem + s * STAGE_BYTES;
                    mbar_expect_tx(&full[s], STAGE_A + STAGE_B);
                    const int y = row0 + i * BK;
#pragma unroll
                    for (int p = 0; p < NS; ++p)
#pragma unroll
                        for (int h = 0; h < 2; ++h)
                            tma_load_2d(st + p * APLANE + h * (APLANE / 2), tm[p], item.y * BM + 64 * h, y, &full[s]);
                    // the coefficients' four digit planes: one contiguous 32 KB tile, already in the swizzled layout
                    const long long tile = (long long)item.z * a.nbt + a.gt0[item.x] + i;
                    bulk_load(st + STAGE_A, a.bimg + tile * STAGE_B, STAGE_B, &full[s]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer: A_j x [B_0 .. B_{3-j}] -> levels j..3
            uint32_t idesc[NS];
#pragma unroll
            for (int j = 0; j < NS; ++j) idesc[j] = idesc_bf16_mn(true, (NS - j) * BN, BM);
            int kc = 0, t = 0;
            for (int it = blockIdx.x; it < a.nitems && !*abort_flag; it += gridDim.x, ++t) {
                const int4 item = a.items[it];
                const int nk = nsteps(item);
                int m0, n0;
                item_mn(item, m0, n0);
                const int kvalid = a.L + 1 - m0;  // degrees; the digit image is zero beyond
                const int ab = t & 1;
                if (t >= 2 && !mbar_wait(&acce[ab], ((t >> 1) - 1) & 1, a.err, 22)) {
                    *abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t dbase = tmem + (uint32_t)(ab * ACC);
                bool ok = true;
                for (int i = 0; i < nk; ++i, ++kc) {
                    const int s = kc % STAGES;
                    if (!mbar_wait(&full[s], (kc / STAGES) & 1, a.err, 23)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
                    const int krem = kvalid - i * BK;
                    const int nkk = krem >= BK ? BK / UK : (krem + UK - 1) / UK;
#pragma unroll
                    for (int kk = 0; kk < BK / UK; ++kk) {
                        if (kk >= nkk) break;
                        const uint64_t bd = smem_desc(st + STAGE_A + kk * UK * 2, 16, 1024);
#pragma unroll
                        for (int j = 0; j < NS; ++j) {
                            const uint64_t ad = smem_desc(st + j * APLANE + kk * UK * 128, APLANE / 2, 1024);
                            const bool first = (i == 0) && kk == 0 && j == 0;  // initialises all four levels
                            mma_bf16(dbase + (uint32_t)(j * BN), ad, bd, idesc[j], first ? 0u : 1u);
                        }
                    }
                    mma_commit(&empty[s]);
                }
                mma_commit(&accf[ab]);
                if (!ok) {
                    *abort_flag = 1;
                    ++t;
                    break;
                }
            }
            for (int u = (t >= 2 ? t - 2 : 0); u < t; ++u) mbar_wait(&accf[u & 1], (u >> 1) & 1, a.err, 26);
        }
    } else {
        // ---------------- epilogue (8 warps: two per TMEM lane quarter, each taking half of the columns; thread =
        // one k row)
        const int quarter = warp & 3, half = (warp - 2) >> 2;
        const int r = quarter * 32 + lane;
        const int N = a.N;
        int t = 0;
        for (int it = blockIdx.x; it < a.nitems && !*abort_flag; it += gridDim.x, ++t) {
            const int4 item = a.items[it];
            int m0, n0;
            item_mn(item, m0, n0);
            const GroupPairs P = group_pairs(m0, n0);
            const int k = item.y * BM + r;
            const bool spectral = a.rhi != nullptr;
            long long poff[4];
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                // synthesis: H(m, n) at (m, n) mod N; spectral residual: at the forward place (-m, -n) mod N
                const int mm = spectral ? -P.m[p] : P.m[p], nn = spectral ? -P.n[p] : P.n[p];
                int pi = mm % N; if (pi < 0) pi += N;
                int qi = nn % N; if (qi < 0) qi += N;
                poff[p] = ((long long)pi * N + qi) * N;
            }
            const int et = k < N ? (int)a.et[(long long)item.x * N + k] : 0;
            if (spectral && k < N) {
                // the FFT values this item will read, requested into L2 while its MMAs run
#pragma unroll 1
                for (int fl = half * (FPT / 2); fl < (half + 1) * (FPT / 2); ++fl) {
                    const int f = item.z * FPT + fl;
                    if (f >= a.batch) break;
                    const long long fo = (long long)f * a.fstride + k;
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        if (p >= P.np) break;
                        prefetch_l2(a.rhi + fo + poff[p]);
                        prefetch_l2(a.rlo + fo + poff[p]);
                    }
                }
            }
            const int ab = t & 1;
            if (!mbar_wait(&accf[ab], (t >> 1) & 1, a.err, 25)) {
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(ab * ACC);
#pragma unroll 1
            for (int cc = half * (BN / 32); cc < (half + 1) * (BN / 32); ++cc) {  // 16 columns = 2 functions x 4 pairs x re/im
                uint32_t v[NS][16];
#pragma unroll
                for (int j = 0; j < NS; ++j) tmem_ld16_nowait(trow + (uint32_t)(j * BN + cc * 16), v[j]);
                tmem_wait_ld();
#pragma unroll
                for (int fq = 0; fq < 2; ++fq) {
                    const int f = item.z * FPT + cc * 2 + fq;
                    if (f >= a.batch || k >= N) continue;
                    const long long fo = (long long)f * a.fstride + k;
                    const signed char* eyf = a.ey + ((long long)f * a.ngroups + item.x) * 4;
                    // spectral residual: the function's four pair values, loads in flight together
                    float2 sh[4], sl[4];
                    if (spectral) {
#pragma unroll
                        for (int p = 0; p < 4; ++p) {
                            sh[p] = sl[p] = make_float2(0.f, 0.f);
                            if (p < P.np) {
                                sh[p] = __ldcs(a.rhi + fo + poff[p]);
                                sl[p] = __ldcs(a.rlo + fo + poff[p]);
                            }
                        }
                    }
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        if (p >= P.np) break;
                        const int E = et + (int)eyf[p] - 14;  // units: 2^(E_T - 7) 2^(E_Y - 7)
                        const int cr = fq * 8 + 2 * p;
                        const df32 re = combine_levels(__uint_as_float(v[0][cr]), __uint_as_float(v[1][cr]),
                                                       __uint_as_float(v[2][cr]), __uint_as_float(v[3][cr]));
                        const df32 im = combine_levels(__uint_as_float(v[0][cr + 1]), __uint_as_float(v[1][cr + 1]),
                                                       __uint_as_float(v[2][cr + 1]), __uint_as_float(v[3][cr + 1]));
                        if (spectral) {
                            // N^2 H = FFT of the synthesised grid; hi - N^2 H.h is exact (close values)
                            const int E2 = E + a.e2n;
                            const float2 h = sh[p], l = sl[p];
                            __stcs(a.rhi + fo + poff[p],
                                   make_float2((h.x - ldexpf(re.h, E2)) + (l.x - ldexpf(re.l, E2)),
                                               (h.y - ldexpf(im.h, E2)) + (l.y - ldexpf(im.l, E2))));
                        } else {
                            a.pout[fo + poff[p]] =
                                make_float4(ldexpf(re.h, E), ldexpf(re.l, E), ldexpf(im.h, E), ldexpf(im.l, E));
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[ab]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ---- plan-time table digits (FP64 arithmetic, once per plan)

__device__ __forceinline__ int exp_above(double mx)
{
    if (!(mx > 0.0)) return EXP_MIN;
    int e;
    frexp(mx, &e);  // mx = m 2^e, m in [0.5, 1): mx < 2^e
    return e < EXP_MIN ? EXP_MIN : (e > EXP_MAX ? EXP_MAX : e);
}

// E_T[g][k]: max over the group's degrees of |d^l(beta_k)| < 2^E_T
__global__ void table_exp_kernel(const double* __restrict__ table, const long long* __restrict__ goff, int L, int N,
                                 int ngroups, signed char* __restrict__ et)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)ngroups * N) return;
    const int g = (int)(idx / N), k = (int)(idx % N);
    int m0, n0;
    group_mn(g, m0, n0);
    const double* tg = table + goff[g] + k;
    double mx = 0.0;
    for (int j = 0; j <= L - m0; ++j) mx = fmax(mx, fabs(tg[(long long)j * N]));
    et[idx] = (signed char)exp_above(mx);
}

// digit planes [row][Kp] of d 2^-E_T: one block per group, rows grow0[g] + j
__global__ void table_digits_kernel(const double* __restrict__ table, const long long* __restrict__ goff, int L, int N,
                                    int Kp, const signed char* __restrict__ et, __nv_bfloat16* __restrict__ p0,
                                    __nv_bfloat16* __restrict__ p1, __nv_bfloat16* __restrict__ p2,
                                    __nv_bfloat16* __restrict__ p3)
{
    const int g = blockIdx.x;
    int m0, n0;
    group_mn(g, m0, n0);
    const int nl = L + 1 - m0;
    const long long row0 = goff[g] / N;
    const double* tg = table + goff[g];
    for (long long e = threadIdx.x; e < (long long)nl * Kp; e += blockDim.x) {
        const int j = (int)(e / Kp), k = (int)(e % Kp);
        double s[NS] = {0.0, 0.0, 0.0, 0.0};
        if (k < N) {
            const double x = ldexp(tg[(long long)j * N + k], -(int)et[(long long)g * N + k]);
            double rr = x * 128.0;
            s[0] = rint(rr);
            rr -= s[0];
            for (int i = 1; i < NS; ++i) {
                rr *= 256.0;
                s[i] = rint(rr);
                rr -= s[i];
            }
        }
        const long long o = (row0 + j) * Kp + k;
        p0[o] = __double2bfloat16(s[0]);
        p1[o] = __double2bfloat16(s[1]);
        p2[o] = __double2bfloat16(s[2]);
        p3[o] = __double2bfloat16(s[3]);
    }
}

// ---- per-call kernels

// the Nyquist pencils (p = B or q = B), which no (m, n) with |m|, |n| <= L maps to
__global__ void zero_nyquist_kernel(float4* __restrict__ H, int N, long long nb)
{
    const long long NN = (long long)N * N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nb * 2 * NN) return;
    const long long f = idx / (2 * NN), r = idx % (2 * NN);
    const int B = N / 2;
    long long o;
    if (r < NN)
        o = (long long)B * NN + r;                            // p = B: [q][k]
    else
        o = ((r - NN) / N) * NN + (long long)B * N + (r - NN) % N;  // q = B: [p][k]
    H[f * NN * N + o] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// r[fn][k][j1][j2] = f - g with g[fn][j1][j2][k] the double-float grid: (f - g.h) - g.l in FP32 (f - g.h is
// exact where g is close to f).  32 x 32 tiles of (k, j2) through shared memory; REAL: real samples and the real
// part of g.  f may be r itself (each element is read and then written by the same thread).
template <bool REAL>
__global__ void __launch_bounds__(256) resid_kernel(const float4* __restrict__ g, const void* fin, float* r, int N)
{
    __shared__ float4 tile[32][33];
    const int k0 = blockIdx.x * 32, q0 = blockIdx.y * 32;
    const long long fj = blockIdx.z;  // fn N + j1
    const long long f = fj / N, j1 = fj % N;
    const long long NN = (long long)N * N;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int y = ty; y < 32; y += 8) {
        const int q = q0 + y, k = k0 + tx;
        if (q < N && k < N) tile[y][tx] = g[f * NN * N + (j1 * N + q) * N + k];
    }
    __syncthreads();
    for (int y = ty; y < 32; y += 8) {
        const int k = k0 + y, q = q0 + tx;
        if (q >= N || k >= N) continue;
        const float4 v = tile[tx][y];
        const long long o = f * NN * N + (long long)k * NN + j1 * N + q;
        if (REAL) {
            r[o] = (((const float*)fin)[o] - v.x) - v.y;
        } else {
            const float2 s = ((const float2*)fin)[o];
            r[2 * o] = (s.x - v.x) - v.y;
            r[2 * o + 1] = (s.y - v.z) - v.w;
        }
    }
}

// The coefficient runs of the contraction: (2l+1) sign F(l, pair) for l = m0..L, as double-float (for FP32 input
// the product is exact: h = fl(c v), l = fma(c, v, -h)).  F packed, or (GROUP) already group-major -- the forward
// GEMM's output, runs at goff2[g] + pair nl + (l - m0).
template <typename CIN, bool GROUP>
__device__ __forceinline__ float4 run_value(const CIN* __restrict__ Fb, long long go, int l, int m0, int nl, int p,
                                            int pm, int pn, int psign)
{
    const CIN v = GROUP ? Fb[go + (long long)p * nl + (l - m0)] : Fb[so3_idx(l, pm, pn)];
    df32 re, im;
    if constexpr (sizeof(v.x) == 8) {
        re = df32((double)(2 * l + 1) * (double)v.x);
        im = df32((double)(2 * l + 1) * (double)v.y);
    } else {
        const float c = (float)(2 * l + 1);
        const float rh = c * (float)v.x, ih = c * (float)v.y;
        re = df32(rh, fmaf(c, (float)v.x, -rh));
        im = df32(ih, fmaf(c, (float)v.y, -ih));
    }
    if (psign < 0) {
        re = -re;
        im = -im;
    }
    return make_float4(re.h, re.l, im.h, im.l);
}

// The coefficients' digit image: for column tile z (functions 8z .. 8z + 7) and group g, the B operand of each
// of the group's K steps (BK degrees) as the contraction's shared-memory stage expects it -- four BF16 digit
// planes of 64 columns (function fl, pair pp, re / im: column 8 fl + 2 pp + {0, 1}) x BK degrees, K-major, each
// column's 128-byte row with its 16-byte chunks swizzled (chunk q at q ^ (row & 7)) -- so that one bulk copy
// fills a stage.  Degrees past the group's run, missing pairs and functions past nb are zero.  One CTA per
// (group, column tile), thread = (column pair c, chunk q8): a first sweep over the run finds the pair's exponent
// E (max |value| < 2^E, written to ey), a second forms the digits of value 2^-E.
template <typename CIN, bool GROUP>
__global__ void __launch_bounds__(256) digit_image_kernel(const CIN* __restrict__ F, long long cstride,
                                                          signed char* __restrict__ ey,
                                                          const long long* __restrict__ goff2,
                                                          const int* __restrict__ gt0, unsigned char* __restrict__ img,
                                                          long long nbt, int L, int ngroups, int nb)
{
    const int g = blockIdx.x, z = blockIdx.y;
    int m0, n0;
    group_mn(g, m0, n0);
    const GroupPairs P = group_pairs(m0, n0);
    const int c = threadIdx.x >> 3, q8 = threadIdx.x & 7;
    const int fl = c >> 2, pp = c & 3, f = z * FPT + fl;
    const int lim = L + 1 - m0, nk = (lim + BK - 1) / BK;
    const bool valid = f < nb && pp < P.np;
    const CIN* Fb = F + (long long)(valid ? f : 0) * cstride;
    const long long go = goff2[g];
    // the pair's (m, n) and sign, selected without a dynamic index into P (which would live in local memory)
    int pm = P.m[0], pn = P.n[0], psign = P.sign[0];
#pragma unroll
    for (int q = 1; q < 4; ++q)
        if (pp == q) {
            pm = P.m[q];
            pn = P.n[q];
            psign = P.sign[q];
        }
    // exponent of the pair's run (the eight threads of a column pair are adjacent lanes)
    float mx = 0.f;
    if (valid)
        for (int i = 0; i < nk; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int li = i * BK + q8 * 8 + j;
                if (li < lim) {
                    const float4 y = run_value<CIN, GROUP>(Fb, go, m0 + li, m0, lim, pp, pm, pn, psign);
                    mx = fmaxf(mx, fmaxf(fabsf(y.x), fabsf(y.z)));
                }
            }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = EXP_MIN;
    if (mx > 0.f) {
        frexpf(mx, &e);  // mx < 2^e; the low word adds at most half an ulp of mx
        e = e < EXP_MIN ? EXP_MIN : (e > EXP_MAX ? EXP_MAX : e);
    }
    if (f < nb && q8 == 0) ey[((long long)f * ngroups + g) * 4 + pp] = (signed char)e;
    const float sc = valid ? pow2f(-e) : 0.f;
    const int Rre = 2 * c, Rim = Rre + 1;
    const uint32_t ore = (uint32_t)Rre * 128u + (uint32_t)((q8 ^ (Rre & 7)) * 16);
    const uint32_t oim = (uint32_t)Rim * 128u + (uint32_t)((q8 ^ (Rim & 7)) * 16);
    for (int i = 0; i < nk; ++i) {
        float4 v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int li = i * BK + q8 * 8 + j;
            v[j] = (valid && li < lim) ? run_value<CIN, GROUP>(Fb, go, m0 + li, m0, lim, pp, pm, pn, psign)
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        uint32_t wre[NS][4], wim[NS][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float dr0[NS], dr1[NS], di0[NS], di1[NS];
            digits4(v[2 * j].x, v[2 * j].y, sc, dr0);
            digits4(v[2 * j + 1].x, v[2 * j + 1].y, sc, dr1);
            digits4(v[2 * j].z, v[2 * j].w, sc, di0);
            digits4(v[2 * j + 1].z, v[2 * j + 1].w, sc, di1);
#pragma unroll
            for (int p = 0; p < NS; ++p) {
                wre[p][j] = pack_bf16(dr0[p], dr1[p]);
                wim[p][j] = pack_bf16(di0[p], di1[p]);
            }
        }
        unsigned char* tile = img + ((long long)z * nbt + gt0[g] + i) * STAGE_B;
#pragma unroll
        for (int p = 0; p < NS; ++p) {
            *reinterpret_cast<uint4*>(tile + p * BPLANE + ore) = make_uint4(wre[p][0], wre[p][1], wre[p][2], wre[p][3]);
            *reinterpret_cast<uint4*>(tile + p * BPLANE + oim) = make_uint4(wim[p][0], wim[p][1], wim[p][2], wim[p][3]);
        }
    }
}

// The synthesis itself, rounded once: grid[fn][k][j1][j2] = the double-float g (complex64, or the real part as
// float32 when REAL), transposed like resid_kernel.
template <bool REAL>
__global__ void __launch_bounds__(256) synth_out_kernel(const float4* __restrict__ g, void* out, int N)
{
    __shared__ float4 tile[32][33];
    const int k0 = blockIdx.x * 32, q0 = blockIdx.y * 32;
    const long long fj = blockIdx.z;  // fn N + j1
    const long long f = fj / N, j1 = fj % N;
    const long long NN = (long long)N * N;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int y = ty; y < 32; y += 8) {
        const int q = q0 + y, k = k0 + tx;
        if (q < N && k < N) tile[y][tx] = g[f * NN * N + (j1 * N + q) * N + k];
    }
    __syncthreads();
    for (int y = ty; y < 32; y += 8) {
        const int k = k0 + y, q = q0 + tx;
        if (q >= N || k >= N) continue;
        const float4 v = tile[tx][y];
        const long long o = f * NN * N + (long long)k * NN + j1 * N + q;
        if (REAL)
            reinterpret_cast<float*>(out)[o] = v.x + v.y;
        else
            reinterpret_cast<float2*>(out)[o] = make_float2(v.x + v.y, v.z + v.w);
    }
}

}  // namespace oz

// --------------------------------------------------------------- host side

using namespace oz;

struct OZState {
    int L = 0, N = 0, B = 0, ngroups = 0, chunk = 0, ntiles = 0, nsm = 0, Kp = 0;
    int pen_fns = 0;  // functions the double-float pencil buffer holds
    long long total_rows = 0, C = 0;
    __nv_bfloat16* planes[NS] = {nullptr, nullptr, nullptr, nullptr};
    CUtensorMap tm[NS];
    signed char* et = nullptr;  // [group][k]
    signed char* ey = nullptr;  // [chunk][group][pair]
    unsigned char* bimg = nullptr;  // [column tile][tile] x STAGE_B: their digit image (digit_image_kernel)
    int* gt0 = nullptr;             // first image tile of each group
    long long nbt = 0;              // image tiles per column tile
    float4* pen = nullptr;      // [chunk][N^3] double-float pencils / grid
    long long* goff2 = nullptr;
    int4* items = nullptr;      // work items of a full chunk (all column tiles)
    int2* iaux = nullptr;
    int nitems = 0;
    // the same lists restricted to the first z column tiles (z = 1 .. ntiles - 1; order kept), for shorter chunks
    std::vector<int4*> items_z;
    std::vector<int2*> iaux_z;
    std::vector<int> nitems_z;
    FFTFactors fac;
    const double* d_tw = nullptr;
    int* err = nullptr;
    long long bytes = 0;
    // exact inverse into host memory: the copy stream and its events (created on first use)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_ready[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr}, ev_join = nullptr;
    unsigned long long ring_seq = 0;  // pieces sent through the ring so far (its slot alternation)
};

bool oz_supported(int L, int N) { return L >= 0 && L <= 255 && N == 2 * (L + 1); }

static int oz_alloc(OZState* o, void** p, size_t bytes, std::string& err)
{
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        err = std::string("cudaMalloc (refinement state): ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? FFTSO3_ERR_OOM : FFTSO3_ERR_CUDA;
    }
    o->bytes += (long long)bytes;
    return FFTSO3_SUCCESS;
}

void oz_destroy(OZState* o)
{
    if (!o) return;
    for (int p = 0; p < NS; ++p)
        if (o->planes[p]) cudaFree(o->planes[p]);
    void* ptrs[] = {o->et, o->ey, o->bimg, o->gt0, o->pen, o->goff2, o->items, o->iaux, o->err};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    for (void* q : o->items_z)
        if (q) cudaFree(q);
    for (void* q : o->iaux_z)
        if (q) cudaFree(q);
    for (cudaEvent_t e : {o->ev_ready[0], o->ev_ready[1], o->ev_free[0], o->ev_free[1], o->ev_join})
        if (e) cudaEventDestroy(e);
    if (o->side) cudaStreamDestroy(o->side);
    delete o;
}

long long oz_device_bytes(const OZState* o) { return o ? o->bytes : 0; }

int oz_create(OZState** out, const double* d_table, const std::vector<long long>& goff, int L, int N, int chunk,
              int pen_fns, const double* d_tw, std::string& err)
{
    *out = nullptr;
    if (!oz_supported(L, N) || chunk < 1 || pen_fns < 1) {
        err = "internal: exact refinement inverse needs SO(3) l_max <= 255";
        return FFTSO3_ERR_UNSUPPORTED;
    }
    OZState* o = new OZState();
    o->L = L;
    o->B = L + 1;
    o->N = N;
    o->ngroups = o->B * o->B;
    o->chunk = chunk;
    o->pen_fns = pen_fns;
    o->ntiles = (chunk + FPT - 1) / FPT;
    o->Kp = (N + 63) / 64 * 64;
    o->C = so3_off(o->B);
    o->total_rows = goff[o->ngroups] / N;
    o->d_tw = d_tw;
    make_fft_factors(N, o->fac);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&o->nsm, cudaDevAttrMultiProcessorCount, dev);
    int rc;
    auto bail = [&](int code) {
        oz_destroy(o);
        return code;
    };
    // exponents and digit planes of the table, from the FP64 table
    long long* d_goff = nullptr;
    if ((rc = oz_alloc(o, (void**)&d_goff, sizeof(long long) * goff.size(), err))) return bail(rc);
    cudaMemcpy(d_goff, goff.data(), sizeof(long long) * goff.size(), cudaMemcpyHostToDevice);
    const size_t plane = sizeof(__nv_bfloat16) * (size_t)o->total_rows * o->Kp;
    for (int p = 0; p < NS; ++p)
        if ((rc = oz_alloc(o, (void**)&o->planes[p], plane, err))) {
            cudaFree(d_goff);
            return bail(rc);
        }
    if ((rc = oz_alloc(o, (void**)&o->et, (size_t)o->ngroups * N, err))) {
        cudaFree(d_goff);
        return bail(rc);
    }
    {
        const long long tot = (long long)o->ngroups * N;
        table_exp_kernel<<<(unsigned)((tot + 255) / 256), 256>>>(d_table, d_goff, L, N, o->ngroups, o->et);
        table_digits_kernel<<<o->ngroups, 256>>>(d_table, d_goff, L, N, o->Kp, o->et, o->planes[0], o->planes[1],
                                                 o->planes[2], o->planes[3]);
        cudaError_t e = cudaDeviceSynchronize();
        cudaFree(d_goff);
        o->bytes -= (long long)(sizeof(long long) * goff.size());
        if (e != cudaSuccess) {
            err = std::string("refinement table digits: ") + cudaGetErrorString(e);
            return bail(FFTSO3_ERR_CUDA);
        }
    }
    for (int p = 0; p < NS; ++p)
        if (!tc_encode_bf16_2d(&o->tm[p], o->planes[p], o->Kp, o->total_rows, 64, BK)) {
            err = "cuTensorMapEncodeTiled failed (refinement table)";
            return bail(FFTSO3_ERR_CUDA);
        }
    // group-major offsets, work items (ordered by decreasing length), per-item (goff2, first row)
    std::vector<long long> goff2(o->ngroups + 1);
    std::vector<int> gt0(o->ngroups);
    std::vector<int4> items;
    std::vector<int2> aux;
    long long acc2 = 0, acct = 0;
    for (int g = 0; g < o->ngroups; ++g) {
        int m0, n0;
        group_mn(g, m0, n0);
        gt0[g] = (int)acct;
        acct += (o->B - m0 + BK - 1) / BK;
        goff2[g] = acc2;
        acc2 += (long long)group_pairs(m0, n0).np * (o->B - m0);
        for (int nt = 0; nt < o->ntiles; ++nt)
            for (int mt = 0; mt * BM < N; ++mt)
                items.push_back(make_int4(g, mt, nt, (m0 << 16) | (n0 + 32768)));
    }
    goff2[o->ngroups] = acc2;
    if (acc2 != o->C) {
        err = "internal: group-major layout does not cover the coefficients";
        return bail(FFTSO3_ERR_CUDA);
    }
    std::stable_sort(items.begin(), items.end(), [&](const int4& x, const int4& y) { return (x.w >> 16) < (y.w >> 16); });
    aux.resize(items.size());
    for (size_t i = 0; i < items.size(); ++i)
        aux[i] = make_int2((int)goff2[items[i].x], (int)(goff[items[i].x] / N));
    o->nitems = (int)items.size();
    o->nbt = acct;
    if ((rc = oz_alloc(o, (void**)&o->gt0, sizeof(int) * gt0.size(), err))) return bail(rc);
    cudaMemcpy(o->gt0, gt0.data(), sizeof(int) * gt0.size(), cudaMemcpyHostToDevice);
    if ((rc = oz_alloc(o, (void**)&o->goff2, sizeof(long long) * goff2.size(), err))) return bail(rc);
    if ((rc = oz_alloc(o, (void**)&o->items, sizeof(int4) * items.size(), err))) return bail(rc);
    if ((rc = oz_alloc(o, (void**)&o->iaux, sizeof(int2) * aux.size(), err))) return bail(rc);
    cudaMemcpy(o->goff2, goff2.data(), sizeof(long long) * goff2.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(o->items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(o->iaux, aux.data(), sizeof(int2) * aux.size(), cudaMemcpyHostToDevice);
    for (int zt = 1; zt < o->ntiles; ++zt) {
        std::vector<int4> iz;
        std::vector<int2> az;
        for (size_t i = 0; i < items.size(); ++i)
            if (items[i].z < zt) {
                iz.push_back(items[i]);
                az.push_back(aux[i]);
            }
        int4* di = nullptr;
        int2* da = nullptr;
        if ((rc = oz_alloc(o, (void**)&di, sizeof(int4) * iz.size(), err))) return bail(rc);
        o->items_z.push_back(di);
        if ((rc = oz_alloc(o, (void**)&da, sizeof(int2) * az.size(), err))) return bail(rc);
        o->iaux_z.push_back(da);
        o->nitems_z.push_back((int)iz.size());
        cudaMemcpy(di, iz.data(), sizeof(int4) * iz.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(da, az.data(), sizeof(int2) * az.size(), cudaMemcpyHostToDevice);
    }
    // per-chunk buffers
    const size_t grid = (size_t)N * N * N;
    if ((rc = oz_alloc(o, (void**)&o->ey, (size_t)chunk * o->ngroups * 4, err))) return bail(rc);
    if ((rc = oz_alloc(o, (void**)&o->bimg, (size_t)STAGE_B * o->ntiles * o->nbt, err))) return bail(rc);
    if ((rc = oz_alloc(o, (void**)&o->pen, sizeof(float4) * (size_t)pen_fns * grid, err))) return bail(rc);
    if ((rc = oz_alloc(o, (void**)&o->err, sizeof(int), err))) return bail(rc);
    cudaMemset(o->err, 0, sizeof(int));
    cudaError_t e = cudaFuncSetAttribute(oz_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        err = std::string("refinement state: ") + cudaGetErrorString(e);
        return bail(FFTSO3_ERR_CUDA);
    }
    *out = o;
    return FFTSO3_SUCCESS;
}

int oz_status(OZState* o)
{
    int v = 0;
    if (o && o->err) cudaMemcpy(&v, o->err, sizeof(int), cudaMemcpyDeviceToHost);
    return v;
}

#define OZK(call)                                                              \
    do {                                                                       \
        cudaError_t _e = (call);                                               \
        if (_e != cudaSuccess) {                                               \
            err = std::string(#call) + ": " + cudaGetErrorString(_e);          \
            return FFTSO3_ERR_CUDA;                                            \
        }                                                                      \
    } while (0)

// coefficients -> double-float group-major runs and their exponents, then the exact contraction: H into the
// double-float pencils (rhi null), or the spectral residual into rhi
// pen: where the synthesis goes (rhi null): o->pen (pen_fns functions), or a caller's buffer of nb functions
static int oz_contract(OZState* o, const void* F, bool f64, int nb, float2* rhi, const float2* rlo, cudaStream_t st,
                       StageTimer* T, std::string& err, bool group = false, int stage = ST_REF_CONTRACT,
                       float4* pen = nullptr)
{
    if (!pen) pen = o->pen;
    if (nb < 1 || nb > o->chunk || (!rhi && pen == o->pen && nb > o->pen_fns)) {
        err = "internal: refinement chunk larger than its buffers";
        return FFTSO3_ERR_CUDA;
    }
    const int N = o->N, L = o->L;
    const long long NN = (long long)N * N;
    T->begin(ST_REFINE, st);
    {
        const dim3 grid((unsigned)o->ngroups, (unsigned)((nb + FPT - 1) / FPT));
        if (f64)
            digit_image_kernel<double2, false><<<grid, 256, 0, st>>>((const double2*)F, o->C, o->ey, o->goff2, o->gt0,
                                                                     o->bimg, o->nbt, L, o->ngroups, nb);
        else if (group)
            digit_image_kernel<float2, true><<<grid, 256, 0, st>>>((const float2*)F, o->C, o->ey, o->goff2, o->gt0,
                                                                   o->bimg, o->nbt, L, o->ngroups, nb);
        else
            digit_image_kernel<float2, false><<<grid, 256, 0, st>>>((const float2*)F, o->C, o->ey, o->goff2, o->gt0,
                                                                    o->bimg, o->nbt, L, o->ngroups, nb);
        OZK(cudaGetLastError());
        if (!rhi) {
            const long long tot = (long long)nb * 2 * NN;
            zero_nyquist_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(pen, N, nb);
            OZK(cudaGetLastError());
        }
    }
    T->end(st);
    T->begin(stage, st);
    {
        Args a;
        const int zt = (nb + FPT - 1) / FPT;  // column tiles holding the chunk's functions
        a.items = zt < o->ntiles ? o->items_z[zt - 1] : o->items;
        a.iaux = zt < o->ntiles ? o->iaux_z[zt - 1] : o->iaux;
        a.nitems = zt < o->ntiles ? o->nitems_z[zt - 1] : o->nitems;
        a.L = L;
        a.N = N;
        a.batch = nb;
        a.ngroups = o->ngroups;
        a.fstride = NN * N;
        a.bimg = o->bimg;
        a.gt0 = o->gt0;
        a.nbt = o->nbt;
        a.ey = o->ey;
        a.et = o->et;
        a.pout = pen;
        a.rhi = rhi;
        a.rlo = rlo;
        int e2n = 0;
        while ((1LL << e2n) < NN) ++e2n;
        a.e2n = e2n;
        a.err = o->err;
        const int nctas = o->nitems < o->nsm ? o->nitems : o->nsm;
        oz_inv_kernel<<<nctas, THREADS, SMEM_BYTES, st>>>(o->tm[0], o->tm[1], o->tm[2], o->tm[3], a);
        OZK(cudaGetLastError());
    }
    T->end(st);
    return FFTSO3_SUCCESS;
}

bool oz_spectral(const OZState* o) { return o && fft_df32_k_supported(o->N); }

int oz_fft_functions(const OZState* o) { return o ? o->pen_fns : 0; }

int oz_chunk(const OZState* o) { return o ? o->chunk : 0; }

int oz_host_join(OZState* o, cudaStream_t st)
{
    if (!o || !o->side) return FFTSO3_SUCCESS;
    if (cudaEventRecord(o->ev_join, o->side) != cudaSuccess || cudaStreamWaitEvent(st, o->ev_join, 0) != cudaSuccess)
        return FFTSO3_ERR_CUDA;
    return FFTSO3_SUCCESS;
}

long long oz_image_bytes_per_column_tile(int L)
{
    long long t = 0;
    for (int m0 = 0; m0 <= L; ++m0) t += (long long)(2 * m0 + 1) * ((L + 1 - m0 + BK - 1) / BK);
    return t * STAGE_B;
}

int oz_forward_fft(OZState* o, const void* fgrid, bool real, int nb, float2* hi, float2* lo, cudaStream_t st,
                   StageTimer* T, std::string& err)
{
    if (!oz_spectral(o) || nb < 1 || nb > o->pen_fns) {
        err = "internal: double-float forward FFT needs N = 64..512 and nb <= its buffer's functions";
        return FFTSO3_ERR_CUDA;
    }
    T->begin(ST_REF_FFT, st);
    OZK(launch_fft_df32_k_forward(o->pen, o->N, nb, fgrid, real, hi, lo, o->d_tw, st));
    T->end(st);
    return FFTSO3_SUCCESS;
}

int oz_resid_pencils(OZState* o, const void* F, bool f64, int nb, float2* hi, const float2* lo, cudaStream_t st,
                     StageTimer* T, std::string& err, bool group_major)
{
    if (!oz_spectral(o) || (group_major && f64)) {
        err = "internal: spectral residual needs N = 64..512 (group-major input: complex64)";
        return FFTSO3_ERR_CUDA;
    }
    return oz_contract(o, F, f64, nb, hi, lo, st, T, err, group_major);
}

// double-float FFT of the synthesis pencils in o->pen over q (lines (fn, p, k)), then over p (lines (fn, q, k)),
// in place, by the generic line kernels (any N)
static int synth_fft_lines(OZState* o, float4* pen, int nb, cudaStream_t st, std::string& err)
{
    const int N = o->N;
    const long long NN = (long long)N * N;
    {
        FFTLaunch Lq;
        Lq.in = pen;
        Lq.out = pen;
        Lq.fac = o->fac;
        Lq.nlines = (long long)nb * NN;
        Lq.lpb = 8;
        Lq.inner = N;
        Lq.ostride = NN;
        Lq.istride = 1;
        Lq.es = N;
        Lq.tw = o->d_tw;
        Lq.fp64 = false;
        Lq.df32 = true;
        Lq.real_in = false;
        Lq.real_out = false;
        Lq.lines_fastest = true;
        OZK(launch_fft_lines(Lq, st));
        FFTLaunch Lp = Lq;
        Lp.inner = NN;
        Lp.ostride = NN * N;
        Lp.es = NN;
        OZK(launch_fft_lines(Lp, st));
    }
    return FFTSO3_SUCCESS;
}

int oz_inverse_resid(OZState* o, const void* F, bool f64, int nb, const void* fgrid, bool real, float* resid,
                     cudaStream_t st, StageTimer* T, std::string& err)
{
    int rc = oz_contract(o, F, f64, nb, nullptr, nullptr, st, T, err);
    if (rc) return rc;
    const int N = o->N;
    // the grid form serves the sizes the spectral form does not (N not a power of two from 64 to 512)
    T->begin(ST_REF_FFT, st);
    if ((rc = synth_fft_lines(o, o->pen, nb, st, err))) return rc;
    T->end(st);
    // residual against the FP32 samples, transposed back to [fn][k][j1][j2]
    T->begin(ST_REFINE, st);
    {
        dim3 grid((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32), (unsigned)((long long)nb * N));
        if (real)
            resid_kernel<true><<<grid, 256, 0, st>>>(o->pen, fgrid, resid, N);
        else
            resid_kernel<false><<<grid, 256, 0, st>>>(o->pen, fgrid, resid, N);
        OZK(cudaGetLastError());
    }
    T->end(st);
    return FFTSO3_SUCCESS;
}

int oz_inverse_exact(OZState* o, const void* F, bool f64, int nb, void* grid, bool real, cudaStream_t st,
                     StageTimer* T, std::string& err, void* pen_buf, void* host, void* ring, bool join,
                     bool group_major)
{
    float4* pen = pen_buf ? (float4*)pen_buf : o->pen;
    if (group_major && f64) {
        err = "internal: group-major input of the exact inverse is complex64";
        return FFTSO3_ERR_CUDA;
    }
    int rc = oz_contract(o, F, f64, nb, nullptr, nullptr, st, T, err, group_major, ST_INV_CONTRACT, pen);
    if (rc) return rc;
    const int N = o->N;
    const long long G = (long long)N * N * N;
    const size_t gbytes = (size_t)G * (real ? sizeof(float) : sizeof(float2));  // one function's grid
    T->begin(ST_INV_FFT, st);
    if (oz_spectral(o) && host) {
        // into host memory: both passes of each piece of OZ_SYNTH_PIECE functions on st into a slot of the
        // two-slot device ring, then the slot's copy to the host on the copy stream, so the copies (the host link
        // bounds them) run under the FFT of the next pieces; a slot is rewritten once its copy is done
        if (!o->side) {
            OZK(cudaStreamCreateWithFlags(&o->side, cudaStreamNonBlocking));
            for (int i = 0; i < 2; ++i) {
                OZK(cudaEventCreateWithFlags(&o->ev_ready[i], cudaEventDisableTiming));
                OZK(cudaEventCreateWithFlags(&o->ev_free[i], cudaEventDisableTiming));
            }
            OZK(cudaEventCreateWithFlags(&o->ev_join, cudaEventDisableTiming));
        }
        for (int f0 = 0; f0 < nb; f0 += OZ_SYNTH_PIECE) {
            // the ring's slots alternate across calls; a slot's last copy (if any) must be done before it is rewritten
            const int np = nb - f0 < OZ_SYNTH_PIECE ? nb - f0 : OZ_SYNTH_PIECE, sl = (int)(o->ring_seq++ & 1);
            float4* pb = pen + (long long)f0 * G;
            char* rb = (char*)ring + (size_t)sl * OZ_SYNTH_PIECE * gbytes;
            OZK(launch_fft_df32_k_synth_pass(1, pb, N, np, rb, real, o->d_tw, st));
            OZK(cudaStreamWaitEvent(st, o->ev_free[sl], 0));
            OZK(launch_fft_df32_k_synth_pass(2, pb, N, np, rb, real, o->d_tw, st));
            OZK(cudaEventRecord(o->ev_ready[sl], st));
            OZK(cudaStreamWaitEvent(o->side, o->ev_ready[sl], 0));
            OZK(cudaMemcpyAsync((char*)host + (size_t)f0 * gbytes, rb, (size_t)np * gbytes, cudaMemcpyDeviceToHost,
                                o->side));
            OZK(cudaEventRecord(o->ev_free[sl], o->side));
        }
        if (join) {
            OZK(cudaEventRecord(o->ev_join, o->side));
            OZK(cudaStreamWaitEvent(st, o->ev_join, 0));
        }
    } else if (oz_spectral(o)) {
        OZK(launch_fft_df32_k_synth(pen, N, nb, grid, real, o->d_tw, st));
    } else {
        if ((rc = synth_fft_lines(o, pen, nb, st, err))) return rc;
        dim3 g((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32), (unsigned)((long long)nb * N));
        if (real)
            synth_out_kernel<true><<<g, 256, 0, st>>>(pen, grid, N);
        else
            synth_out_kernel<false><<<g, 256, 0, st>>>(pen, grid, N);
        OZK(cudaGetLastError());
        if (host) OZK(cudaMemcpyAsync(host, grid, (size_t)nb * gbytes, cudaMemcpyDeviceToHost, st));
    }
    T->end(st);
    return FFTSO3_SUCCESS;
}

}  // namespace fftso3
