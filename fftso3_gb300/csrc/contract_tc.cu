// Tensor-core beta-sum contraction for SO(3) (FFTSO3_PREC_TC_BF16X3), sm_103a.
//
// The beta-sum of fdcl_FFTSO3.cpp:704-740 and its inverse (grid form of
// :498-531) are, per symmetry group g (m0 >= |n0|, up to 4 (m,n) pairs sharing
// one Wigner-d block), dense products with the group's table block
// D_g[l][k] = d^l_{m0 n0}(beta_k):
//   forward  F_g[l][c] = sum_k D_g[l][k] X_g[k][c],  X_g[k][c] = w_k G_k(pair, fn) re/im
//   inverse  H_g[k][c] = sum_l D_g[l][k] Y_g[l][c],  Y_g[l][c] = (2l+1) sign F(l, pair, fn) re/im
// with c running over (function, pair, re/im): 8 columns per function.
//
// Precision: each operand is split into three BF16 terms (x = x0 + x1 + x2,
// 24 significant bits) and the six products with i + j <= 2 are accumulated
// by tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulator in TMEM).
//
// Kernel structure (one CTA per (group, 128-row tile, 128-column tile)):
//   warp 0: TMA producer (cp.async.bulk.tensor, 128B swizzle) into a 2-stage ring
//   warp 1: TMEM allocator and single-thread tcgen05.mma issuer; tcgen05.commit
//           releases ring slots and finally signals the accumulator
//   warps 2-5: epilogue, tcgen05.ld 32x32b from their TMEM lane quarter, scatter
//           to the coefficient vector (forward) or the grid work buffer (inverse)
// The forward reads the table K-major (k contiguous); the inverse reads the
// same table as an MN-major operand (M = k), so one table serves both.
// Every mbarrier wait is bounded (about one second of clock64 time); on
// timeout the kernel records an error code and unwinds, freeing its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <vector>

#include "../../include/fftso3_gb300.h"
#include "common.cuh"
#include "contract.cuh"
#include "tc.cuh"

namespace fftso3 {

namespace tc {

constexpr int BM = 128;          // MMA M (rows of the accumulator = TMEM lanes)
constexpr int BN = 128;          // MMA N (accumulator columns)
constexpr int BK = 64;           // k-step per ring slot (one 128-byte swizzle row of BF16)
constexpr int UK = 16;           // K per tcgen05.mma (kind::f16)
constexpr int STAGES = 2;
constexpr int PLANE_BYTES = 128 * 128;        // 128 rows x 128 bytes
constexpr int STAGE_BYTES = 6 * PLANE_BYTES;  // 3 A planes + 3 B planes
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*barriers*/ + 1024 /*alignment*/;
constexpr int THREADS = 192;
// TMEM accumulators: k-steps go round-robin to NKC chunk accumulators, and in
// each chunk the leading product (x0 * y0) and the five smaller products
// accumulate separately, so the small terms are never rounded against the
// large running sum.  NACC * BN <= 512 TMEM columns.
constexpr int NKC = 2;
constexpr int NACC = 2 * NKC;
constexpr long long WAIT_CYCLES = 2000000000LL;  // ~1 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false (and an error code in *err) after ~1 s.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code)
{
    if (mbar_try_wait(bar, parity)) return true;
    long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > WAIT_CYCLES) {
            atomicCAS(err, 0, code);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)tm), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// UMMA shared-memory descriptor, 128-byte swizzle (SM100 layout code 2, version 1).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, M = 128, N = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(bool a_mn_major)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn_major ? 1u : 0u) << 15) | ((uint32_t)(BN >> 3) << 17) |
           ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct GemmArgs {
    const int2* items;         // (group, row tile)
    const long long* grow0;    // first table row of each group
    int L, N, ncols, batch;
    int nk_fixed;              // forward: k-steps over the beta axis (Kp / BK)
    long long cstride;         // coefficients per function
    float2* F;                 // forward output coefficients [batch][C]
    float2* H;                 // inverse output work grid [batch][N][N][N]
    int* err;
};

// FWD = true: A = table (K-major, rows l), B = X planes; D[l][c].
// FWD = false: A = table^T (MN-major, rows k), B = Y planes; D[k][c].
template <bool FWD>
__global__ void __launch_bounds__(THREADS, 1)
    so3_tc_gemm_kernel(const __grid_constant__ CUtensorMap tA0, const __grid_constant__ CUtensorMap tA1,
                       const __grid_constant__ CUtensorMap tA2, const __grid_constant__ CUtensorMap tB0,
                       const __grid_constant__ CUtensorMap tB1, const __grid_constant__ CUtensorMap tB2,
                       GemmArgs args)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;
    uint32_t* tmem_slot = (uint32_t*)(accf + 1);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int2 item = args.items[blockIdx.x];
    const int g = item.x, mt = item.y, nt = blockIdx.y;
    int m0, n0;
    group_mn(g, m0, n0);
    const int B = args.L + 1;
    const int nl = B - m0;
    const int nk = FWD ? args.nk_fixed : (nl + BK - 1) / BK;
    const long long row0 = args.grow0[g];

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accf, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(NACC * BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        const CUtensorMap* tA[3] = {&tA0, &tA1, &tA2};
        const CUtensorMap* tB[3] = {&tB0, &tB1, &tB2};
        const int brow = g * args.ncols + nt * BN;
        for (int i = 0; i < nk && !*abort_flag; ++i) {
            const int s = i % STAGES;
            if (i >= STAGES && !mbar_wait(&empty[s], ((i / STAGES) - 1) & 1, args.err, 1)) {
                *abort_flag = 1;
                break;
            }
            unsigned char* st = smem + s * STAGE_BYTES;
            mbar_expect_tx(&full[s], STAGE_BYTES);
            for (int p = 0; p < 3; ++p) {
                unsigned char* a = st + p * PLANE_BYTES;
                if (FWD) {
                    tma_load_2d(a, tA[p], i * BK, (int)(row0 + (long long)mt * BM), &full[s]);
                } else {
                    const int y = (int)(row0 + (long long)i * BK);
                    tma_load_2d(a, tA[p], mt * BM, y, &full[s]);
                    tma_load_2d(a + PLANE_BYTES / 2, tA[p], mt * BM + 64, y, &full[s]);
                }
                tma_load_2d(st + (3 + p) * PLANE_BYTES, tB[p], i * BK, brow, &full[s]);
            }
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        constexpr uint32_t idesc = idesc_bf16(!FWD);
        // products (a, b) with a + b <= 2 of the 3-term splits
        const int pa[6] = {0, 0, 1, 0, 1, 2};
        const int pb[6] = {0, 1, 0, 2, 1, 0};
        for (int i = 0; i < nk; ++i) {
            const int s = i % STAGES;
            if (!mbar_wait(&full[s], (i / STAGES) & 1, args.err, 2)) {
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
            for (int kk = 0; kk < BK / UK; ++kk) {
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    uint64_t ad, bd;
                    const uint32_t abase = st + pa[q] * PLANE_BYTES;
                    const uint32_t bbase = st + (3 + pb[q]) * PLANE_BYTES;
                    if (FWD) {
                        ad = smem_desc(abase + kk * UK * 2, 16, 1024);
                    } else {
                        // MN-major: 64-wide k blocks 8 KB apart (LBO), 8-row l groups 1 KB apart (SBO)
                        ad = smem_desc(abase + kk * UK * 128, PLANE_BYTES / 2, 1024);
                    }
                    bd = smem_desc(bbase + kk * UK * 2, 16, 1024);
                    const int acc = (i % NKC) * 2 + (q == 0 ? 0 : 1);
                    const bool first = (i < NKC) && kk == 0 && (q <= 1);
                    mma_bf16(tmem + (uint32_t)(acc * BN), ad, bd, idesc, first ? 0u : 1u);
                }
            }
            mma_commit(&empty[s]);
        }
        mma_commit(accf);
    } else if (warp >= 2) {
        // ---------------- epilogue
        const int quarter = warp & 3;
        const int r = quarter * 32 + lane;
        const bool ok = mbar_wait(accf, 0, args.err, 3);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (ok) {
            const GroupPairs P = group_pairs(m0, n0);
            const int N = args.N;
            const int nacc = 2 * (nk < NKC ? nk : NKC);
            for (int chunk = 0; chunk < BN / 32; ++chunk) {
                double v[32];
                {
                    float u[32];
                    tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + chunk * 32, u);
#pragma unroll
                    for (int t = 0; t < 32; ++t) v[t] = (double)u[t];
                }
                for (int j = 1; j < nacc; ++j) {
                    float u[32];
                    tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + j * BN + chunk * 32, u);
#pragma unroll
                    for (int t = 0; t < 32; ++t) v[t] += (double)u[t];
                }
#pragma unroll
                for (int fl = 0; fl < 4; ++fl) {
                    const int f = (nt * BN + chunk * 32) / 8 + fl;
                    if (f >= args.batch) continue;
                    if (FWD) {
                        const int l = m0 + mt * BM + r;
                        if (r + mt * BM >= nl) continue;
                        float2* Fo = args.F + (long long)f * args.cstride;
                        for (int p = 0; p < P.np; ++p) {
                            const double sg = P.sign[p];
                            Fo[so3_idx(l, P.m[p], P.n[p])] =
                                make_float2((float)(sg * v[fl * 8 + 2 * p]), (float)(sg * v[fl * 8 + 2 * p + 1]));
                        }
                    } else {
                        const int k = mt * BM + r;
                        if (k >= N) continue;
                        float2* Ho = args.H + (long long)f * N * N * N + (long long)k * N * N;
                        for (int p = 0; p < P.np; ++p) {
                            int pi = P.m[p] % N; if (pi < 0) pi += N;
                            int qi = P.n[p] % N; if (qi < 0) qi += N;
                            Ho[(long long)pi * N + qi] = make_float2((float)v[fl * 8 + 2 * p], (float)v[fl * 8 + 2 * p + 1]);
                        }
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NACC * BN));
    }
}

// ------------------------------------------------------------ pack kernels

__device__ __forceinline__ void split3(double x, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l)
{
    h = __double2bfloat16(x);
    double r = x - (double)__bfloat162float(h);
    m = __double2bfloat16(r);
    r -= (double)__bfloat162float(m);
    l = __double2bfloat16(r);
}

// FP64 table [rows][N] -> three BF16 planes [rows][Kp] (zero for k >= N).
__global__ void table_split_kernel(const double* __restrict__ t, __nv_bfloat16* __restrict__ p0,
                                   __nv_bfloat16* __restrict__ p1, __nv_bfloat16* __restrict__ p2, long long rows,
                                   int N, int Kp)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * Kp) return;
    long long r = i / Kp;
    int k = (int)(i % Kp);
    double x = (k < N) ? t[r * N + k] : 0.0;
    __nv_bfloat16 a, b, c;
    split3(x, a, b, c);
    p0[i] = a;
    p1[i] = b;
    p2[i] = c;
}

// X planes [g * ncols + col][Kp]: col = f*8 + p*2 + (re/im); x = w_k G_k(-m_p, -n_p).
__global__ void pack_fwd_kernel(const float2* __restrict__ G, const double* __restrict__ w,
                                __nv_bfloat16* __restrict__ x0, __nv_bfloat16* __restrict__ x1,
                                __nv_bfloat16* __restrict__ x2, int L, int N, int Kp, int ncols, int batch,
                                int ngroups)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)ngroups * ncols * Kp;
    if (i >= total) return;
    int k = (int)(i % Kp);
    long long rc = i / Kp;
    int col = (int)(rc % ncols);
    int g = (int)(rc / ncols);
    int f = col / 8, p = (col % 8) / 2, ri = col & 1;
    int m0, n0;
    group_mn(g, m0, n0);
    GroupPairs P = group_pairs(m0, n0);
    double x = 0.0;
    if (k < N && f < batch && p < P.np) {
        int pi = (-P.m[p]) % N; if (pi < 0) pi += N;
        int qi = (-P.n[p]) % N; if (qi < 0) qi += N;
        float2 v = G[(long long)f * N * N * N + (long long)k * N * N + (long long)pi * N + qi];
        x = w[k] * (double)(ri ? v.y : v.x);
    }
    __nv_bfloat16 a, b, c;
    split3(x, a, b, c);
    x0[i] = a;
    x1[i] = b;
    x2[i] = c;
}

// Y planes [g * ncols + col][KLp]: y = (2l+1) sign_p F(l, m_p, n_p) re/im, l = m0 + l'.
__global__ void pack_inv_kernel(const float2* __restrict__ F, __nv_bfloat16* __restrict__ y0,
                                __nv_bfloat16* __restrict__ y1, __nv_bfloat16* __restrict__ y2, int L, int KLp,
                                int ncols, int batch, int ngroups, long long cstride)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)ngroups * ncols * KLp;
    if (i >= total) return;
    int lp = (int)(i % KLp);
    long long rc = i / KLp;
    int col = (int)(rc % ncols);
    int g = (int)(rc / ncols);
    int f = col / 8, p = (col % 8) / 2, ri = col & 1;
    int m0, n0;
    group_mn(g, m0, n0);
    GroupPairs P = group_pairs(m0, n0);
    int l = m0 + lp;
    double y = 0.0;
    if (l <= L && f < batch && p < P.np) {
        float2 v = F[(long long)f * cstride + so3_idx(l, P.m[p], P.n[p])];
        y = (double)(2 * l + 1) * P.sign[p] * (double)(ri ? v.y : v.x);
    }
    __nv_bfloat16 a, b, c;
    split3(y, a, b, c);
    y0[i] = a;
    y1[i] = b;
    y2[i] = c;
}

}  // namespace tc

// --------------------------------------------------------------- host side

using namespace tc;

struct TCState {
    int L = 0, B = 0, N = 0, Kp = 0, KLp = 0, batch = 0, ncols = 0, ngroups = 0;
    bool refine = false;
    FFTFactors fac;
    const double* d_tw = nullptr;
    const double* d_w = nullptr;
    long long total_rows = 0;
    __nv_bfloat16* d_tab[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16* d_x[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16* d_y[3] = {nullptr, nullptr, nullptr};
    float2* d_work = nullptr;
    float2* d_resid = nullptr;   // refinement: residual grid
    float2* d_coef2 = nullptr;   // refinement: correction coefficients
    long long* d_grow0 = nullptr;
    int2* d_items_fwd = nullptr;
    int2* d_items_inv = nullptr;
    int n_items_fwd = 0, n_items_inv = 0;
    CUtensorMap tmA_fwd[3], tmA_inv[3], tmX[3], tmY[3];
    int* d_err = nullptr;
    long long bytes = 0;
};

// cuTensorMapEncodeTiled is resolved through the runtime's driver entry-point
// query, so the library does not link libcuda directly.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

static bool encode_2d(CUtensorMap* tm, const void* base, unsigned long long inner, unsigned long long outer,
                      unsigned box_inner, unsigned box_outer)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * 2};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims,
                                        strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

static int tc_alloc(TCState* s, void** p, size_t bytes, std::string& err)
{
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        err = std::string("cudaMalloc (tensor-core state): ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? FFTSO3_ERR_OOM : FFTSO3_ERR_CUDA;
    }
    s->bytes += (long long)bytes;
    return FFTSO3_SUCCESS;
}

void tc_destroy(TCState* s)
{
    if (!s) return;
    for (int p = 0; p < 3; ++p) {
        if (s->d_tab[p]) cudaFree(s->d_tab[p]);
        if (s->d_x[p]) cudaFree(s->d_x[p]);
        if (s->d_y[p]) cudaFree(s->d_y[p]);
    }
    void* ptrs[] = {s->d_work, s->d_resid, s->d_coef2, s->d_grow0, s->d_items_fwd, s->d_items_inv, s->d_err};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    delete s;
}

long long tc_device_bytes(const TCState* s) { return s ? s->bytes : 0; }

int tc_create(TCState** out, int L, int N, int batch, const double* d_table_fp64, const std::vector<long long>& goff,
              long long table_elems, const double* d_tw, const double* d_w, const FFTFactors& fac, bool refine,
              std::string& err)
{
    *out = nullptr;
    TCState* s = new TCState();
    s->L = L;
    s->B = L + 1;
    s->N = N;
    s->Kp = (N + 63) / 64 * 64;
    s->KLp = (s->B + 63) / 64 * 64;
    s->batch = batch;
    s->ncols = (8 * batch + BN - 1) / BN * BN;
    s->ngroups = s->B * s->B;
    s->refine = refine;
    s->fac = fac;
    s->d_tw = d_tw;
    s->d_w = d_w;
    s->total_rows = table_elems / N;
    int rc;
    auto bail = [&](int code) {
        tc_destroy(s);
        return code;
    };
    // table planes
    for (int p = 0; p < 3; ++p)
        if ((rc = tc_alloc(s, (void**)&s->d_tab[p], sizeof(__nv_bfloat16) * s->total_rows * s->Kp, err)))
            return bail(rc);
    {
        long long tot = s->total_rows * s->Kp;
        table_split_kernel<<<(unsigned)((tot + 255) / 256), 256>>>(d_table_fp64, s->d_tab[0], s->d_tab[1],
                                                                   s->d_tab[2], s->total_rows, N, s->Kp);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            err = std::string("table split: ") + cudaGetErrorString(e);
            return bail(FFTSO3_ERR_CUDA);
        }
    }
    const size_t xelems = (size_t)s->ngroups * s->ncols * s->Kp;
    const size_t yelems = (size_t)s->ngroups * s->ncols * s->KLp;
    for (int p = 0; p < 3; ++p) {
        if ((rc = tc_alloc(s, (void**)&s->d_x[p], sizeof(__nv_bfloat16) * xelems, err))) return bail(rc);
        if ((rc = tc_alloc(s, (void**)&s->d_y[p], sizeof(__nv_bfloat16) * yelems, err))) return bail(rc);
    }
    const size_t gridel = (size_t)batch * N * N * N;
    if ((rc = tc_alloc(s, (void**)&s->d_work, sizeof(float2) * gridel, err))) return bail(rc);
    if (refine) {
        if ((rc = tc_alloc(s, (void**)&s->d_resid, sizeof(float2) * gridel, err))) return bail(rc);
        if ((rc = tc_alloc(s, (void**)&s->d_coef2, sizeof(float2) * (size_t)batch * so3_off(s->B), err)))
            return bail(rc);
    }
    // group rows and work items
    std::vector<long long> grow0(s->ngroups);
    std::vector<int2> itf, iti;
    for (int g = 0; g < s->ngroups; ++g) {
        int m0, n0;
        group_mn(g, m0, n0);
        grow0[g] = goff[g] / N;
        int nl = s->B - m0;
        for (int mt = 0; mt * BM < nl; ++mt) itf.push_back(make_int2(g, mt));
        for (int mt = 0; mt * BM < N; ++mt) iti.push_back(make_int2(g, mt));
    }
    s->n_items_fwd = (int)itf.size();
    s->n_items_inv = (int)iti.size();
    if ((rc = tc_alloc(s, (void**)&s->d_grow0, sizeof(long long) * grow0.size(), err))) return bail(rc);
    if ((rc = tc_alloc(s, (void**)&s->d_items_fwd, sizeof(int2) * itf.size(), err))) return bail(rc);
    if ((rc = tc_alloc(s, (void**)&s->d_items_inv, sizeof(int2) * iti.size(), err))) return bail(rc);
    if ((rc = tc_alloc(s, (void**)&s->d_err, sizeof(int), err))) return bail(rc);
    cudaMemcpy(s->d_grow0, grow0.data(), sizeof(long long) * grow0.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(s->d_items_fwd, itf.data(), sizeof(int2) * itf.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(s->d_items_inv, iti.data(), sizeof(int2) * iti.size(), cudaMemcpyHostToDevice);
    cudaMemset(s->d_err, 0, sizeof(int));
    // tensor maps
    for (int p = 0; p < 3; ++p) {
        bool ok = encode_2d(&s->tmA_fwd[p], s->d_tab[p], s->Kp, s->total_rows, 64, BM) &&
                  encode_2d(&s->tmA_inv[p], s->d_tab[p], s->Kp, s->total_rows, 64, BK) &&
                  encode_2d(&s->tmX[p], s->d_x[p], s->Kp, (unsigned long long)s->ngroups * s->ncols, 64, BN) &&
                  encode_2d(&s->tmY[p], s->d_y[p], s->KLp, (unsigned long long)s->ngroups * s->ncols, 64, BN);
        if (!ok) {
            err = "cuTensorMapEncodeTiled failed";
            return bail(FFTSO3_ERR_CUDA);
        }
    }
    cudaError_t e = cudaFuncSetAttribute(so3_tc_gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SMEM_BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(so3_tc_gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) {
        err = std::string("tensor-core kernel attributes: ") + cudaGetErrorString(e);
        return bail(FFTSO3_ERR_CUDA);
    }
    *out = s;
    return FFTSO3_SUCCESS;
}

static FFTLaunch fft_launch(const TCState* s, const void* in, void* out, bool cols)
{
    FFTLaunch L;
    const int N = s->N;
    L.in = in;
    L.out = out;
    L.fac = s->fac;
    L.tw = s->d_tw;
    L.fp64 = false;
    L.real_in = false;
    L.real_out = false;
    if (!cols) {
        L.nlines = (long long)s->batch * N * N;
        L.lpb = 4;
        L.inner = 1;
        L.ostride = N;
        L.istride = 0;
        L.es = 1;
        L.lines_fastest = false;
    } else {
        L.nlines = (long long)s->batch * N * N;
        L.lpb = 16;
        L.inner = N;
        L.ostride = (long long)N * N;
        L.istride = 1;
        L.es = N;
        L.lines_fastest = true;
    }
    return L;
}

#define TCK(call)                                                          \
    do {                                                                   \
        cudaError_t _e = (call);                                           \
        if (_e != cudaSuccess) {                                           \
            err = std::string(#call) + ": " + cudaGetErrorString(_e);      \
            return FFTSO3_ERR_CUDA;                                        \
        }                                                                  \
    } while (0)

static int tc_forward_once(TCState* s, const float2* grid, float2* F, cudaStream_t st, StageTimer* T,
                           std::string& err)
{
    const int N = s->N;
    T->begin(ST_FFT_ROWS, st);
    TCK(launch_fft_lines(fft_launch(s, grid, s->d_work, false), st));
    T->end(st);
    T->begin(ST_FFT_COLS, st);
    TCK(launch_fft_lines(fft_launch(s, s->d_work, s->d_work, true), st));
    T->end(st);
    {
        T->begin(ST_PACK_FWD, st);
        long long tot = (long long)s->ngroups * s->ncols * s->Kp;
        pack_fwd_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(s->d_work, s->d_w, s->d_x[0], s->d_x[1],
                                                                        s->d_x[2], s->L, N, s->Kp, s->ncols, s->batch,
                                                                        s->ngroups);
        TCK(cudaGetLastError());
        T->end(st);
    }
    GemmArgs a;
    a.items = s->d_items_fwd;
    a.grow0 = s->d_grow0;
    a.L = s->L;
    a.N = N;
    a.ncols = s->ncols;
    a.batch = s->batch;
    a.nk_fixed = s->Kp / BK;
    a.cstride = so3_off(s->B);
    a.F = F;
    a.H = nullptr;
    a.err = s->d_err;
    dim3 lg(s->n_items_fwd, s->ncols / BN);
    T->begin(ST_GEMM_FWD, st);
    so3_tc_gemm_kernel<true><<<lg, THREADS, SMEM_BYTES, st>>>(s->tmA_fwd[0], s->tmA_fwd[1], s->tmA_fwd[2], s->tmX[0],
                                                                s->tmX[1], s->tmX[2], a);
    TCK(cudaGetLastError());
    T->end(st);
    return FFTSO3_SUCCESS;
}

static int tc_inverse_once(TCState* s, const float2* F, float2* grid, cudaStream_t st, StageTimer* T,
                           std::string& err)
{
    const int N = s->N;
    {
        T->begin(ST_PACK_INV, st);
        long long tot = (long long)s->ngroups * s->ncols * s->KLp;
        pack_inv_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(F, s->d_y[0], s->d_y[1], s->d_y[2], s->L,
                                                                        s->KLp, s->ncols, s->batch, s->ngroups,
                                                                        so3_off(s->B));
        TCK(cudaGetLastError());
        T->end(st);
    }
    T->begin(ST_NYQUIST, st);
    TCK(launch_zero_nyquist_so3(s->d_work, false, N, (long long)s->batch * N, st));
    T->end(st);
    GemmArgs a;
    a.items = s->d_items_inv;
    a.grow0 = s->d_grow0;
    a.L = s->L;
    a.N = N;
    a.ncols = s->ncols;
    a.batch = s->batch;
    a.nk_fixed = 0;
    a.cstride = so3_off(s->B);
    a.F = nullptr;
    a.H = s->d_work;
    a.err = s->d_err;
    dim3 lg(s->n_items_inv, s->ncols / BN);
    T->begin(ST_GEMM_INV, st);
    so3_tc_gemm_kernel<false><<<lg, THREADS, SMEM_BYTES, st>>>(s->tmA_inv[0], s->tmA_inv[1], s->tmA_inv[2],
                                                                 s->tmY[0], s->tmY[1], s->tmY[2], a);
    TCK(cudaGetLastError());
    T->end(st);
    T->begin(ST_FFT_ROWS, st);
    TCK(launch_fft_lines(fft_launch(s, s->d_work, s->d_work, false), st));
    T->end(st);
    T->begin(ST_FFT_COLS, st);
    TCK(launch_fft_lines(fft_launch(s, s->d_work, grid, true), st));
    T->end(st);
    return FFTSO3_SUCCESS;
}

__global__ void resid_kernel(const float2* __restrict__ f, float2* __restrict__ r, long long n)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 a = f[i], b = r[i];
    r[i] = make_float2(a.x - b.x, a.y - b.y);
}

__global__ void add_kernel(float2* __restrict__ F, const float2* __restrict__ d, long long n)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2 a = F[i], b = d[i];
    F[i] = make_float2(a.x + b.x, a.y + b.y);
}

int tc_forward(TCState* s, const void* grid, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    int rc = tc_forward_once(s, (const float2*)grid, (float2*)coeffs, st, T, err);
    if (rc || !s->refine) return rc;
    // one residual step: F += forward(f - inverse(F))
    const long long ng = (long long)s->batch * s->N * s->N * s->N;
    const long long nc = (long long)s->batch * so3_off(s->B);
    if ((rc = tc_inverse_once(s, (const float2*)coeffs, s->d_resid, st, T, err))) return rc;
    T->begin(ST_REFINE, st);
    resid_kernel<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>((const float2*)grid, s->d_resid, ng);
    TCK(cudaGetLastError());
    T->end(st);
    if ((rc = tc_forward_once(s, s->d_resid, s->d_coef2, st, T, err))) return rc;
    T->begin(ST_REFINE, st);
    add_kernel<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>((float2*)coeffs, s->d_coef2, nc);
    TCK(cudaGetLastError());
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_inverse(TCState* s, const void* coeffs, void* grid, cudaStream_t st, StageTimer* T, std::string& err)
{
    return tc_inverse_once(s, (const float2*)coeffs, (float2*)grid, st, T, err);
}

int tc_status(TCState* s)
{
    int h = 0;
    if (cudaMemcpy(&h, s->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h;
}

}  // namespace fftso3
