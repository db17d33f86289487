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
// Data path.  The 2-D FFT output is transposed to k-contiguous pencils
// G'[fn][p][q][k], so each (function, pair) column of X_g is one contiguous
// run.  The GEMM is persistent (one CTA per SM walking a work list of
// (group, row tile, column tile) items) and warp-specialised:
//   warp 0     TMA producer of the table tiles (cp.async.bulk.tensor, 128-byte
//              swizzle; the three BF16 planes of the table are precomputed);
//   warp 1     TMEM owner and single-thread tcgen05.mma issuer;
//   warps 2-5  B-operand producers: gather X (pencils) or Y (coefficients)
//              in FP32, split each value into three BF16 terms and store them
//              straight into the swizzled shared-memory tile;
//   warps 6-9  epilogue: tcgen05.ld from a double-buffered TMEM accumulator,
//              then the forward scatters coefficients and the inverse writes
//              k-contiguous pencils H'[fn][p][q][k] (coalesced).
// The forward reads the table K-major (k contiguous); the inverse reads the
// same table as an MN-major operand (M = k), so one table serves both.
// All arithmetic in these kernels is FP32/BF16 (the FP64 pipe is slow on this
// part).  Every mbarrier wait is bounded (about one second of clock64 time);
// on timeout the kernel records an error code and unwinds, freeing its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/fftso3_gb300.h"
#include "common.cuh"
#include "contract.cuh"
#include "fused.cuh"
#include "tc.cuh"
#include "tc_ptx.cuh"

namespace fftso3 {

namespace tc {

using namespace ptx;

constexpr int BM = 128;          // MMA M (rows of the accumulator = TMEM lanes)
constexpr int BN = 128;          // MMA N (accumulator columns = 16 functions x 4 pairs x re/im)
constexpr int FPT = BN / 8;      // SO(3): functions per column tile (4 (m,n) pairs x re/im each)
constexpr int FPT_S2 = BN / 4;   // S^2: functions per column tile (pairs m, -m x re/im)
constexpr int BK = 64;           // k-step per ring slot (one 128-byte swizzle row of BF16)
constexpr int UK = 16;           // K per tcgen05.mma (kind::f16)
constexpr int STAGES = 2;
constexpr int PLANE_BYTES = 128 * 128;        // 128 rows x 128 bytes
constexpr int STAGE_A = 3 * PLANE_BYTES;      // three BF16 planes of the table tile (TMA)
constexpr int STAGE_BYTES = 6 * PLANE_BYTES;  // + three planes of the B tile (producer warps)
constexpr int NPROD = 8;                      // B-producer warps
constexpr int NEPI = 4;                       // epilogue warps
constexpr int THREADS = 32 * (2 + NPROD + NEPI);
constexpr int MAXN = 1024;                    // weights staged in shared memory
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 256 /*barriers*/ + 4 * MAXN /*weights*/ + 1024 /*alignment*/;
// TMEM: two accumulator buffers (double-buffered across work items); in each
// the leading product (x0 * y0) and the five smaller products accumulate in
// separate 128-column halves, so the small terms are never rounded against
// the large running sum.
constexpr int TMEM_COLS = 512;

// k-steps of table tiles the forward GEMM prefetches into L2 ahead of its TMA ring.
#ifndef FFTSO3_GEMM_PF
#define FFTSO3_GEMM_PF 3
#endif

// Instruction descriptor of this kernel's tiles (M = m, N = n; defaults BM x BN).
__host__ __device__ constexpr uint32_t idesc_bf16(bool a_mn_major, int n = BN, int m = BM)
{
    return idesc_bf16_mn(a_mn_major, n, m);
}

// 1: a forward row tile with at most 64 valid rows (degrees) issues M = 64 MMAs
// (half the tensor work of the padded 128-row tile).  Their accumulator rows
// r < 64 sit in TMEM lanes 32 (r / 16) + r % 16 (16 lanes of each 32-lane
// quarter), which the epilogue reads accordingly.
#ifndef FFTSO3_MMA_M64
#define FFTSO3_MMA_M64 1
#endif

// 1: the products A_hi B_hi (-> hi accumulator) and A_hi B_mid (-> lo accumulator)
// are one N = 256 MMA over the adjacent B_hi and B_mid planes into the
// adjacent hi and lo accumulators (5 MMA instructions per 16-wide k instead of 6).
#ifndef FFTSO3_MMA_N256
#define FFTSO3_MMA_N256 1
#endif
// hi + lo accumulator columns [c, c + 32): both loads in flight, one wait.
__device__ __forceinline__ void tmem_ld32_one(uint32_t t, float* v)
{
    uint32_t a[32];
    tmem_ld32_nowait(t, a);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(a[i]);
}

__device__ __forceinline__ void tmem_ld32_sum(uint32_t thi, uint32_t tlo, float* v)
{
    uint32_t a[32], b[32];
    tmem_ld32_nowait(thi, a);
    tmem_ld32_nowait(tlo, b);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(a[i]) + __uint_as_float(b[i]);
}

__device__ __forceinline__ void split3f(float x, uint16_t& h, uint16_t& m, uint16_t& l)
{
    __nv_bfloat16 a = __float2bfloat16_rn(x);
    float r = x - __bfloat162float(a);
    __nv_bfloat16 b = __float2bfloat16_rn(r);
    r -= __bfloat162float(b);
    __nv_bfloat16 c = __float2bfloat16_rn(r);
    h = __bfloat16_as_ushort(a);
    m = __bfloat16_as_ushort(b);
    l = __bfloat16_as_ushort(c);
}

// split3f of two values at once, packed as BF16 pairs (x0 in the low half):
// one cvt.rn.bf16x2.f32 per term, the BF16 -> FP32 widening by shifts.  The
// same roundings as split3f, so the same bits.
__device__ __forceinline__ void split3f_pair(float x0, float x1, uint32_t& h, uint32_t& m, uint32_t& l)
{
    auto pack = [](float a, float b) {
        const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);  // .x = a (low half), .y = b
        return *reinterpret_cast<const uint32_t*>(&v);
    };
    h = pack(x0, x1);
    const float r0 = x0 - __uint_as_float(h << 16), r1 = x1 - __uint_as_float(h & 0xffff0000u);
    m = pack(r0, r1);
    const float s0 = r0 - __uint_as_float(m << 16), s1 = r1 - __uint_as_float(m & 0xffff0000u);
    l = pack(s0, s1);
}

struct GemmArgs {
    const int4* items;         // (group, row tile, column tile, -)
    const int2* iaux;          // per item: (group-major offset goff2[g], first table row grow0[g])
    int nitems;
    int csize;                 // CTAs per cluster sharing each table tile (items in blocks of csize)
    const long long* grow0;    // first table row of each group
    int L, N, Kp, batch;
    long long fstride;         // pencil elements per function (N^3)
    long long cstride;         // coefficients per function
    const long long* goff2;    // group-major coefficient offsets: sum over earlier groups of np * nl
    const float2* pin;         // forward: input pencils G'[fn][p][q][k]
    const float2* cin;         // inverse: scaled group-major coefficients Y[fn][goff2 + pair * nl + l']
    float2* cout;              // forward: group-major output coefficients [fn][goff2 + pair * nl + l']
    float2* pout;              // inverse: output pencils H'[fn][p][q][k]
    const float* wf;           // forward: quadrature weights (FP32)
    int* err;
};

// One plan's share of a fused launch over several plans (the l_max buckets of
// an uneven batch): its table maps and arguments.  Work items of a fused launch
// carry (segment << 16 | column tile) in .z.
struct GemmSeg {  // aligned as CUtensorMap (128 bytes), as TMA needs for maps in global memory
    CUtensorMap tm[3];
    GemmArgs a;
};

// Work items carry (group, row tile, column tile, m0 << 16 | (n0 + 32768)).
__host__ __device__ __forceinline__ int item_w(int m0, int n0) { return (m0 << 16) | (n0 + 32768); }
__device__ __forceinline__ void item_mn(const int4& it, int& m0, int& n0)
{
    m0 = it.w >> 16;
    n0 = (it.w & 0xFFFF) - 32768;
}

// One-term form: the BF16 rounding of 8 consecutive k values into row R of plane 0 only.
__device__ __forceinline__ void store_chunk1(uint32_t bplanes, int R, int chunk, const float* x8)
{
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const __nv_bfloat162 v = __floats2bfloat162_rn(x8[2 * j], x8[2 * j + 1]);  // .x = low half
        w[j] = *reinterpret_cast<const uint32_t*>(&v);
    }
    const uint32_t off = (uint32_t)R * 128u + (uint32_t)((chunk ^ (R & 7)) * 16);
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(bplanes + off), "r"(w[0]), "r"(w[1]), "r"(w[2]),
                 "r"(w[3])
                 : "memory");
}

// Store 8 consecutive k values (one 16-byte chunk) of row R of each BF16 plane.
__device__ __forceinline__ void store_chunk(uint32_t bplanes, int R, int chunk, const float* x8)
{
    uint32_t w[3][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) split3f_pair(x8[2 * j], x8[2 * j + 1], w[0][j], w[1][j], w[2][j]);
    const uint32_t off = (uint32_t)R * 128u + (uint32_t)((chunk ^ (R & 7)) * 16);
#pragma unroll
    for (int pl = 0; pl < 3; ++pl) {
        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(bplanes + pl * PLANE_BYTES + off),
                     "r"(w[pl][0]), "r"(w[pl][1]), "r"(w[pl][2]), "r"(w[pl][3])
                     : "memory");
    }
}

// S^2 groups: g = m >= 0, pair 0 = (m, FFT bin m), pair 1 = (-m, bin N - m)
// with sign (-1)^m (fdcl_FFTS2.cpp:160-166); the inverse writes pair 0 to bin
// -m mod N and pair 1 to bin m (f = sum_m H(m) e^{+i m phi} by a forward DFT).
__device__ __forceinline__ GroupPairs s2_pairs(int m)
{
    GroupPairs p;
    p.np = m > 0 ? 2 : 1;
    p.m[0] = m;
    p.n[0] = 0;
    p.sign[0] = 1;
    p.m[1] = -m;
    p.n[1] = 0;
    p.sign[1] = (m & 1) ? -1 : 1;
    p.m[2] = p.m[3] = p.n[2] = p.n[3] = 0;
    p.sign[2] = p.sign[3] = 1;
    return p;
}

// FWD = true: A = table (K-major, rows l), B = X from pencils; D[l][c].
// FWD = false: A = table^T (MN-major, rows k), B = Y from coefficients; D[k][c].
// S2 = false: SO(3) Wigner-d groups, pencils [fn][p][q][k], 4 pairs per function;
// S2 = true: S^2 Legendre groups (g = m), pencils [fn][p][k], 2 pairs per function.
// FUSED = true: the work list spans several plans (segments); each item's
// table map, sizes and buffers come from segs[item.z >> 16] (args then holds
// only the merged item list and the error word).
// args.csize = C > 1: the launch is in clusters of C CTAs and the work list in
// blocks of C items with the same (group, row tile) and consecutive column
// tiles; the C CTAs of a cluster take one block together, each table tile is
// read once for all of them (each CTA issues its share of the tile's TMA boxes
// with cluster multicast) and a stage is released when all C CTAs' MMAs are
// done with it (multicast commits; empty barriers count C).
// TERMS: BF16 terms per operand, 3 (split-BF16, six products) or 1 (one product: a refinement's correction,
// whose input is small, needs no more)
template <bool FWD, bool S2, bool FUSED, int TERMS = 3>
__global__ void __launch_bounds__(THREADS, 1)
    so3_tc_gemm_kernel(const __grid_constant__ CUtensorMap tA0, const __grid_constant__ CUtensorMap tA1,
                       const __grid_constant__ CUtensorMap tA2, const __grid_constant__ GemmArgs args,
                       const GemmSeg* __restrict__ segs)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;
    uint64_t* acce = accf + 2;
    uint32_t* tmem_slot = (uint32_t*)(acce + 2);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
    float* wsm = (float*)(smem + STAGES * STAGE_BYTES + 256);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int PPF = S2 ? 2 : 4;        // pairs per function
    constexpr int FPTK = BN / (2 * PPF);   // functions per column tile
    // per-item arguments and column tile
    auto argsof = [&](const int4& it) -> const GemmArgs& { return FUSED ? segs[it.z >> 16].a : args; };
    auto ctile = [&](const int4& it) { return FUSED ? (it.z & 0xFFFF) : it.z; };
    auto nsteps = [&](const int4& it, const GemmArgs& A) {
        int m0, n0;
        item_mn(it, m0, n0);
        return FWD ? A.Kp / BK : (A.L + 1 - m0 + BK - 1) / BK;
    };

    const int CL = FUSED ? 1 : args.csize;
    const uint32_t crank = CL > 1 ? cluster_rank() : 0;
    const uint16_t cmask = (uint16_t)((1u << CL) - 1u);
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1 + NPROD);
            mbar_init(&empty[s], CL);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], NEPI);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (FWD && !FUSED)
        for (int i = threadIdx.x; i < args.N; i += THREADS) wsm[i] = args.wf[i];
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (CL > 1) cluster_sync();  // every CTA's barriers initialised before any multicast reaches them
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- TMA producer of the table tiles
            // The ring holds only STAGES k-steps, so each step's tiles are also
            // prefetched into L2 PF steps ahead (across item boundaries): the
            // table streams from HBM with more bytes in flight than the ring.
            constexpr int PF = FWD ? FFTSO3_GEMM_PF : 0;  // the inverse re-reads each table tile from L2 (4 row tiles)
            auto prefetch = [&](int it, int i) {
                while (PF > 0 && it < args.nitems) {
                    const int4 item = args.items[it];
                    const GemmArgs& A = argsof(item);
                    const int nk = nsteps(item, A);
                    if (i < nk) {
                        const long long row0 = args.iaux[it].y;
                        for (int p = 0; p < TERMS; ++p) {
                            const CUtensorMap* tm = FUSED ? &segs[item.z >> 16].tm[p] : (p == 0 ? &tA0 : p == 1 ? &tA1 : &tA2);
                            if (FWD) {
                                if (p % CL == (int)crank) tma_prefetch_2d(tm, i * BK, (int)(row0 + (long long)item.y * BM));
                            } else {
                                const int y = (int)(row0 + (long long)i * BK);
                                if ((2 * p) % CL == (int)crank) tma_prefetch_2d(tm, item.y * BM, y);
                                if ((2 * p + 1) % CL == (int)crank) tma_prefetch_2d(tm, item.y * BM + 64, y);
                            }
                        }
                        return;
                    }
                    i -= nk;
                    it += gridDim.x;
                }
            };
            for (int i = 0; i < PF; ++i) prefetch(blockIdx.x, i);
            int kc = 0;
            int4 nitem = make_int4(0, 0, 0, 0);
            int nrow0 = 0;
            if (blockIdx.x < args.nitems) {
                nitem = args.items[blockIdx.x];
                nrow0 = args.iaux[blockIdx.x].y;
            }
            for (int it = blockIdx.x; it < args.nitems && !*abort_flag; it += gridDim.x) {
                const int4 item = nitem;
                const long long row0 = nrow0;
                if (it + (int)gridDim.x < args.nitems) {  // one item ahead
                    nitem = args.items[it + gridDim.x];
                    nrow0 = args.iaux[it + gridDim.x].y;
                }
                const GemmArgs& A = argsof(item);
                const CUtensorMap* tA[3] = {FUSED ? &segs[item.z >> 16].tm[0] : &tA0,
                                            FUSED ? &segs[item.z >> 16].tm[1] : &tA1,
                                            FUSED ? &segs[item.z >> 16].tm[2] : &tA2};
                const int nk = nsteps(item, A);
                for (int i = 0; i < nk; ++i, ++kc) {
                    prefetch(it, i + PF);
                    const int s = kc % STAGES;
                    if (kc >= STAGES && !mbar_wait(&empty[s], ((kc / STAGES) - 1) & 1, args.err, 1)) {
                        *abort_flag = 1;
                        break;
                    }
                    unsigned char* st = smem + s * STAGE_BYTES;
                    // the whole tile (its planes) lands in every CTA of the cluster
                    mbar_expect_tx(&full[s], TERMS * PLANE_BYTES);
                    // the tile's boxes: plane p (forward), or plane p half h (inverse) = box j = 2 p + h;
                    // box j is issued by cluster rank j mod C
                    for (int p = 0; p < TERMS; ++p) {
                        unsigned char* a = st + p * PLANE_BYTES;
                        if (FWD) {
                            if (p % CL != (int)crank) continue;
                            if (CL > 1)
                                tma_load_2d_mc(a, tA[p], i * BK, (int)(row0 + (long long)item.y * BM), &full[s], cmask);
                            else
                                tma_load_2d(a, tA[p], i * BK, (int)(row0 + (long long)item.y * BM), &full[s]);
                        } else {
                            const int y = (int)(row0 + (long long)i * BK);
                            for (int h = 0; h < 2; ++h) {
                                if ((2 * p + h) % CL != (int)crank) continue;
                                if (CL > 1)
                                    tma_load_2d_mc(a + h * (PLANE_BYTES / 2), tA[p], item.y * BM + 64 * h, y, &full[s],
                                                   cmask);
                                else
                                    tma_load_2d(a + h * (PLANE_BYTES / 2), tA[p], item.y * BM + 64 * h, y, &full[s]);
                            }
                        }
                    }
                }
            }
            // cluster: the last stages' tiles (this CTA's boxes and the other CTAs' multicasts) have
            // landed in this CTA before the cluster's final barrier lets any CTA exit
            if (CL > 1)
                for (int k = (kc > STAGES ? kc - STAGES : 0); k < kc; ++k)
                    mbar_wait(&full[k % STAGES], (k / STAGES) & 1, args.err, 7);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer
            constexpr uint32_t idesc = idesc_bf16(!FWD);
            constexpr uint32_t idesc256 = idesc_bf16(!FWD, 2 * BN);
            constexpr uint32_t idesc_h = idesc_bf16(!FWD, BN, BM / 2);
            constexpr uint32_t idesc256_h = idesc_bf16(!FWD, 2 * BN, BM / 2);
            const int pa[6] = {0, 0, 1, 0, 1, 2};
            const int pb[6] = {0, 1, 0, 2, 1, 0};
            int kc = 0, t = 0;
            int4 nitem = blockIdx.x < args.nitems ? args.items[blockIdx.x] : make_int4(0, 0, 0, 0);
            for (int it = blockIdx.x; it < args.nitems && !*abort_flag; it += gridDim.x, ++t) {
                const int4 item = nitem;
                if (it + (int)gridDim.x < args.nitems) nitem = args.items[it + gridDim.x];  // one item ahead
                const GemmArgs& A = argsof(item);
                const int nk = nsteps(item, A);
                int m0, n0;
                item_mn(item, m0, n0);
                // valid K (zero-padded beyond): the forward sums over N samples, the inverse over nl degrees;
                // the last k-step issues only the 16-wide MMAs that hold valid K
                const int kvalid = FWD ? A.N : A.L + 1 - m0;
                const bool half = FWD && FFTSO3_MMA_M64 && (A.L + 1 - m0 - item.y * BM) <= BM / 2;
                const uint32_t id1 = half ? idesc_h : idesc, id2 = half ? idesc256_h : idesc256;
                const int ab = t & 1;
                if (t >= 2 && !mbar_wait(&acce[ab], ((t >> 1) - 1) & 1, args.err, 2)) {
                    *abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t dhi = tmem + (uint32_t)(ab * 256), dlo = dhi + 128;
                bool ok = true;
                for (int i = 0; i < nk; ++i, ++kc) {
                    const int s = kc % STAGES;
                    if (!mbar_wait(&full[s], (kc / STAGES) & 1, args.err, 3)) {
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
#pragma unroll
                        for (int q = 0; q < (TERMS == 3 ? 6 : 1); ++q) {
                            if (TERMS == 3 && FFTSO3_MMA_N256 && q == 1) continue;  // issued with q = 0
                            const uint32_t abase = st + pa[q] * PLANE_BYTES;
                            const uint32_t bbase = st + STAGE_A + pb[q] * PLANE_BYTES;
                            const uint64_t ad = FWD ? smem_desc(abase + kk * UK * 2, 16, 1024)
                                                    : smem_desc(abase + kk * UK * 128, PLANE_BYTES / 2, 1024);
                            const uint64_t bd = smem_desc(bbase + kk * UK * 2, 16, 1024);
                            const bool first = (i == 0) && kk == 0 && q <= 1;
                            mma_bf16(q == 0 ? dhi : dlo, ad, bd, (TERMS == 3 && FFTSO3_MMA_N256 && q == 0) ? id2 : id1,
                                     first ? 0u : 1u);
                        }
                    }
                    if (CL > 1)
                        mma_commit_mc(&empty[s], cmask);  // the stage's table tile is shared by the cluster
                    else
                        mma_commit(&empty[s]);
                }
                mma_commit(&accf[ab]);
                if (!ok) {
                    *abort_flag = 1;
                    ++t;
                    break;
                }
            }
            // the accumulator commits of the last item(s) must land before TMEM is freed
            for (int u = (t >= 2 ? t - 2 : 0); u < t; ++u) mbar_wait(&accf[u & 1], (u >> 1) & 1, args.err, 6);
        }
    } else if (warp < 2 + NPROD) {
        // ---------------- B-operand producers (256 threads): thread = (column pair, k quarter q4),
        // covering the 16-byte chunks q4 and q4 + 4 of each 64-wide k-step (so the
        // swizzled stores of a warp spread over all eight bank groups).  Each
        // k-step's loads are issued one step ahead into registers so the DRAM
        // latency overlaps the split/store of the previous step.
        const int pt = threadIdx.x - 64;
        const int c = pt >> 2, q4 = pt & 3;
        // odd columns store their two chunks in the opposite order, so the 8 threads of a quarter-warp
        // (2 columns x 4 chunks) cover all 8 16-byte bank groups of the swizzled rows
        const int hs = c & 1;
        const int fl = c / PPF, pp = c % PPF;
        const int Rre = fl * 2 * PPF + 2 * pp, Rim = Rre + 1;
        struct Src {
            const float2* p;  // run start for this (function, pair), or null
            int lim;          // valid extent of the run (N, or nl)
            int N;            // the item's grid size (weights are zero beyond it)
            const float* wf;  // the item's quadrature weights (fused launches)
        };
        auto source = [&](const int4& item, const int2& aux) -> Src {
            const GemmArgs& A = argsof(item);
            const int N = A.N;
            int m0, n0;
            item_mn(item, m0, n0);
            const GroupPairs P = S2 ? s2_pairs(m0) : group_pairs(m0, n0);
            const int f = ctile(item) * FPTK + fl;
            Src r;
            r.lim = FWD ? N : A.L + 1 - m0;
            r.N = N;
            r.wf = A.wf;
            r.p = nullptr;
            if (f >= A.batch || pp >= P.np) return r;
            if (FWD && S2) {
                const int bin = pp == 0 ? m0 : N - m0;
                r.p = A.pin + (long long)f * A.fstride + (long long)bin * N;
            } else if (FWD) {
                int pi = (-P.m[pp]) % N; if (pi < 0) pi += N;
                int qi = (-P.n[pp]) % N; if (qi < 0) qi += N;
                r.p = A.pin + (long long)f * A.fstride + ((long long)pi * N + qi) * N;
            } else {
                r.p = A.cin + (long long)f * A.cstride + aux.x + (long long)pp * r.lim;
            }
            return r;
        };
        auto fetch = [&](const Src& sr, int i, float2* v) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = i * BK + (q4 + 4 * (h ^ hs)) * 8;
                if (FWD && sr.p && k + 8 <= sr.lim) {
                    const float4* s4 = reinterpret_cast<const float4*>(sr.p + k);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        float4 t = __ldg(s4 + j);
                        v[8 * h + 2 * j] = make_float2(t.x, t.y);
                        v[8 * h + 2 * j + 1] = make_float2(t.z, t.w);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        v[8 * h + j] = (sr.p && k + j < sr.lim) ? __ldg(sr.p + k + j) : make_float2(0.f, 0.f);
                }
            }
        };
        int kc = 0;
        int it = blockIdx.x, i = 0;
        float2 cur[16];
        Src scur, snxt;
        int nk_cur = 0;
        // the next item's metadata is loaded one item ahead (no dependent load at a transition)
        int4 pitem = make_int4(0, 0, 0, 0);
        int2 paux = make_int2(0, 0);
        if (it < args.nitems) {
            const int4 item0 = args.items[it];
            scur = source(item0, args.iaux[it]);
            nk_cur = nsteps(item0, argsof(item0));
            fetch(scur, 0, cur);
            if (it + (int)gridDim.x < args.nitems) {
                pitem = args.items[it + gridDim.x];
                paux = args.iaux[it + gridDim.x];
            }
        }
        while (it < args.nitems && !*abort_flag) {
            int it2 = it, i2 = i + 1, nk2 = nk_cur;
            snxt = scur;
            if (i2 == nk_cur) {
                it2 += gridDim.x;
                i2 = 0;
                if (it2 < args.nitems) {
                    snxt = source(pitem, paux);
                    nk2 = nsteps(pitem, argsof(pitem));
                    if (it2 + (int)gridDim.x < args.nitems) {
                        pitem = args.items[it2 + gridDim.x];
                        paux = args.iaux[it2 + gridDim.x];
                    }
                }
            }
            float2 nxt[16];
            if (it2 < args.nitems) fetch(snxt, i2, nxt);
            if (FWD && it2 < args.nitems && snxt.p) {
                // pencil runs two k-steps further into L2 (the register prefetch covers one)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int k = (i2 + 2) * BK + (q4 + 4 * h) * 8;
                    if (k < snxt.lim) asm volatile("prefetch.global.L2 [%0];" ::"l"(snxt.p + k) : "memory");
                }
            }
            const int s = kc % STAGES;
            if (kc >= STAGES && !mbar_wait(&empty[s], ((kc / STAGES) - 1) & 1, args.err, 4)) {
                *abort_flag = 1;
                break;
            }
            const uint32_t bpl = smem_u32(smem + s * STAGE_BYTES + STAGE_A);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int chunk = q4 + 4 * (h ^ hs);
                const int k = i * BK + chunk * 8;
                float re[8], im[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const float2 v = cur[h * 8 + j];
                    const float wk =
                        FWD ? ((k + j < scur.N) ? (FUSED ? __ldg(scur.wf + k + j) : wsm[k + j]) : 0.f) : 1.f;
                    re[j] = v.x * wk;
                    im[j] = v.y * wk;
                }
                if constexpr (TERMS == 3) {
                    store_chunk(bpl, Rre, chunk, re);
                    store_chunk(bpl, Rim, chunk, im);
                } else {
                    store_chunk1(bpl, Rre, chunk, re);
                    store_chunk1(bpl, Rim, chunk, im);
                }
            }
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) mbar_arrive(&full[s]);
#pragma unroll
            for (int j = 0; j < 16; ++j) cur[j] = nxt[j];
            scur = snxt;
            nk_cur = nk2;
            it = it2;
            i = i2;
            ++kc;
        }
    } else {
        // ---------------- epilogue (4 warps, one TMEM lane quarter each)
        const int quarter = warp & 3;
        const int r = quarter * 32 + lane;
        int t = 0;
        int4 nitem = make_int4(0, 0, 0, 0);
        int2 naux = make_int2(0, 0);
        if (blockIdx.x < args.nitems) {
            nitem = args.items[blockIdx.x];
            naux = args.iaux[blockIdx.x];
        }
        for (int it = blockIdx.x; it < args.nitems && !*abort_flag; it += gridDim.x, ++t) {
            const int4 item = nitem;
            const int2 aux = naux;
            if (it + (int)gridDim.x < args.nitems) {  // one item ahead
                nitem = args.items[it + gridDim.x];
                naux = args.iaux[it + gridDim.x];
            }
            const GemmArgs& A = argsof(item);
            const int N = A.N;
            int m0, n0;
            item_mn(item, m0, n0);
            const GroupPairs P = S2 ? s2_pairs(m0) : group_pairs(m0, n0);
            const int nl = A.L + 1 - m0;
            const bool half = FWD && FFTSO3_MMA_M64 && (nl - item.y * BM) <= BM / 2;  // M = 64 item (see MMA)
            long long poff[4];
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                if (FWD) {
                    poff[p] = aux.x + (long long)p * nl;
                } else if (S2) {
                    int bin = (p == 0 ? -m0 : m0) % N; if (bin < 0) bin += N;
                    poff[p] = (long long)bin * N;
                } else {
                    int pi = P.m[p] % N; if (pi < 0) pi += N;
                    int qi = P.n[p] % N; if (qi < 0) qi += N;
                    poff[p] = ((long long)pi * N + qi) * N;
                }
            }
            const int ab = t & 1;
            if (!mbar_wait(&accf[ab], (t >> 1) & 1, args.err, 5)) {
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(ab * 256);
            for (int chunk = 0; chunk < BN / 32; ++chunk) {
                float v[32];
                if constexpr (TERMS == 3) tmem_ld32_sum(trow + chunk * 32, trow + 128 + chunk * 32, v);
                else tmem_ld32_one(trow + chunk * 32, v);
#pragma unroll
                for (int fq = 0; fq < 32 / (2 * PPF); ++fq) {
                    const int f = ctile(item) * FPTK + chunk * (32 / (2 * PPF)) + fq;
                    if (f >= A.batch) continue;
                    if (FWD) {
                        // M = 64 tiles: rows 16 quarter + lane (lanes 0..15 of each quarter)
                        const int row = half ? item.y * BM + quarter * 16 + lane : item.y * BM + r;
                        if ((half && lane >= 16) || row >= nl) continue;
                        float2* Fo = A.cout + (long long)f * A.cstride + row;
#pragma unroll
                        for (int p = 0; p < 4; ++p) {
                            if (p >= P.np) break;
                            const float sg = (float)P.sign[p];
                            Fo[poff[p]] = make_float2(sg * v[fq * 2 * PPF + 2 * p], sg * v[fq * 2 * PPF + 2 * p + 1]);
                        }
                    } else {
                        const int k = item.y * BM + r;
                        if (k >= N) continue;
                        float2* Ho = A.pout + (long long)f * A.fstride + k;
#pragma unroll
                        for (int p = 0; p < 4; ++p) {
                            if (p >= P.np) break;
                            Ho[poff[p]] = make_float2(v[fq * 2 * PPF + 2 * p], v[fq * 2 * PPF + 2 * p + 1]);
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
    if (CL > 1) cluster_sync();  // no CTA exits while another may still multicast into it or arrive on its barriers
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ------------------------------------------------- FP32 (CUDA-core) form
//
// The same products on the FP32 pipes (FFTSO3_PREC_FP32): one CTA of 256
// threads per work item (group, row tile, column tile) computes the 128 x 128
// tile D[rows][c] = sum over K of A[rows][K] B[K][c] with FP32 FMAs, 8 x 8
// outputs per thread, K in steps of 16 staged in shared memory.  A comes from
// an FP32 copy of the table ([row][Kp], zero for k >= N), read K-major for the
// forward (rows l, K = k) and transposed for the inverse (rows k, K = l); B is
// X (pencils x weights) or Y (group-major coefficients), as in the
// tensor-core kernel, and so are the epilogue's scatters.
constexpr int SBK = 16;

template <bool FWD, bool S2>
__global__ void __launch_bounds__(256) so3_fp32_gemm_kernel(const float* __restrict__ tab, GemmArgs args)
{
    __shared__ __align__(16) float As[SBK][BM + 4];
    __shared__ __align__(16) float Bs[SBK][BN + 4];
    constexpr int PPF = S2 ? 2 : 4;
    constexpr int FPTK = BN / (2 * PPF);
    const int B = args.L + 1, N = args.N, Kp = args.Kp;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int4 item = args.items[blockIdx.x];
    int m0, n0;
    item_mn(item, m0, n0);
    const GroupPairs P = S2 ? s2_pairs(m0) : group_pairs(m0, n0);
    const int nl = B - m0;
    const long long row0 = args.grow0[item.x];
    const int K = FWD ? N : nl;
    const int mbase = item.y * BM;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < K; k0 += SBK) {
        // A tile
        for (int e = threadIdx.x; e < BM * SBK; e += 256) {
            float v;
            if (FWD) {
                const int i = e / SBK, kk = e - i * SBK;
                const int m = mbase + i, k = k0 + kk;
                v = (m < nl && k < N) ? __ldg(tab + (row0 + m) * Kp + k) : 0.f;
                As[kk][i] = v;
            } else {
                const int kk = e / BM, i = e - kk * BM;
                const int l = k0 + kk, k = mbase + i;
                v = (l < nl && k < N) ? __ldg(tab + (row0 + l) * Kp + k) : 0.f;
                As[kk][i] = v;
            }
        }
        // B tile: 64 (function, pair) columns x re/im
        for (int e = threadIdx.x; e < (BN / 2) * SBK; e += 256) {
            const int cp = e / SBK, kk = e - cp * SBK;
            const int fl = cp / PPF, pp = cp % PPF;
            const int f = item.z * FPTK + fl, k = k0 + kk;
            float2 v = make_float2(0.f, 0.f);
            if (f < args.batch && pp < P.np && k < K) {
                if (FWD) {
                    long long off;
                    if (S2) {
                        const int bin = pp == 0 ? m0 : N - m0;
                        off = (long long)bin * N;
                    } else {
                        int pi = (-P.m[pp]) % N; if (pi < 0) pi += N;
                        int qi = (-P.n[pp]) % N; if (qi < 0) qi += N;
                        off = ((long long)pi * N + qi) * N;
                    }
                    v = __ldg(args.pin + (long long)f * args.fstride + off + k);
                    const float wk = __ldg(args.wf + k);
                    v.x *= wk;
                    v.y *= wk;
                } else {
                    v = __ldg(args.cin + (long long)f * args.cstride + args.goff2[item.x] + (long long)pp * nl + k);
                }
            }
            Bs[kk][2 * cp] = v.x;
            Bs[kk][2 * cp + 1] = v.y;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < SBK; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[kk][ty * 8]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[kk][ty * 8 + 4]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 8]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 8 + 4]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    // epilogue: thread columns tx*8 .. tx*8+7 = (function, pair) tx*4 .. tx*4+3, re/im
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
        const int cp = tx * 4 + jj;
        const int fl = cp / PPF, pp = cp % PPF;
        const int f = item.z * FPTK + fl;
        if (f >= args.batch || pp >= P.np) continue;
        long long base;
        if (FWD) {
            base = (long long)f * args.cstride + args.goff2[item.x] + (long long)pp * nl;
        } else if (S2) {
            int bin = (pp == 0 ? -m0 : m0) % N; if (bin < 0) bin += N;
            base = (long long)f * args.fstride + (long long)bin * N;
        } else {
            int pi = P.m[pp] % N; if (pi < 0) pi += N;
            int qi = P.n[pp] % N; if (qi < 0) qi += N;
            base = (long long)f * args.fstride + ((long long)pi * N + qi) * N;
        }
        const float sg = FWD ? (float)P.sign[pp] : 1.f;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int r = mbase + ty * 8 + i;
            if (r >= (FWD ? nl : N)) break;
            const float2 v = make_float2(sg * acc[i][2 * jj], sg * acc[i][2 * jj + 1]);
            if (FWD) args.cout[base + r] = v;
            else args.pout[base + r] = v;
        }
    }
}

// FP64 table [rows][N] -> FP32 [rows][Kp] (zero for k >= N).
__global__ void table_fp32_kernel(const double* __restrict__ t, float* __restrict__ o, long long rows, int N, int Kp)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * Kp) return;
    const long long r = i / Kp;
    const int k = (int)(i % Kp);
    o[i] = (k < N) ? (float)t[r * N + k] : 0.f;
}

// ------------------------------------------------------- helper kernels

// FP64 table [rows][N] -> three BF16 planes [rows][Kp] (zero for k >= N);
// the value is first rounded to FP32, whose 24 bits the three terms carry.
__global__ void table_split_kernel(const double* __restrict__ t, __nv_bfloat16* __restrict__ p0,
                                   __nv_bfloat16* __restrict__ p1, __nv_bfloat16* __restrict__ p2, long long rows,
                                   int N, int Kp)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * Kp) return;
    long long r = i / Kp;
    int k = (int)(i % Kp);
    float x = (k < N) ? (float)t[r * N + k] : 0.f;
    uint16_t a, b, c;
    split3f(x, a, b, c);
    p0[i] = __ushort_as_bfloat16(a);
    p1[i] = __ushort_as_bfloat16(b);
    p2[i] = __ushort_as_bfloat16(c);
}

// Batched 2-D transpose in[nb][R][Cc] -> out[nb][Cc][R] (complex64), 32x32 tiles.
__global__ void transpose_kernel(const float2* __restrict__ in, float2* __restrict__ out, long long R, long long Cc)
{
    __shared__ float2 tile[32][33];
    const long long c0 = (long long)blockIdx.x * 32, r0 = (long long)blockIdx.y * 32;
    const long long boff = (long long)blockIdx.z * R * Cc;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int j = ty; j < 32; j += 8) {
        long long r = r0 + j, c = c0 + tx;
        if (r < R && c < Cc) tile[j][tx] = in[boff + r * Cc + c];
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        long long c = c0 + j, r = r0 + tx;
        if (r < R && c < Cc) out[boff + c * R + r] = tile[tx][j];
    }
}

// Zero the Nyquist pencils (p = B or q = B) of H'[fn][p][q][k].
__global__ void zero_nyquist_pencils_kernel(float2* __restrict__ H, int N, long long nf)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = 2LL * N * N;  // per function: N pencils of each kind, N values each
    if (i >= nf * per) return;
    long long f = i / per, r = i % per;
    const int B = N / 2;
    long long which = r / ((long long)N * N), rr = r % ((long long)N * N);
    long long a = rr / N, k = rr % N;
    long long off = (which == 0) ? (((long long)B * N + a) * N + k) : ((a * N + B) * N + k);
    H[f * (long long)N * N * N + off] = make_float2(0.f, 0.f);
}

// Tiled permutations between the group-major layout (contiguous in l for a
// fixed (m, n)) and the packed layout (contiguous in m for a fixed (l, n)):
// one CTA per (function, n, 32 l's, 32 m's) stages the tile in shared memory,
// so both sides move runs of 32 consecutive elements.  The group of (m, n) has
// m0 = max(|m|, |n|) and rows l = m0..L; the pair index and sign follow
// group_pairs() (pair_of()).
constexpr int PT = 32;

// grid: x = n + L (2L + 1), y = l tile (ceil(B / 32)), z = m tile + mtiles * (function / PFPC).
// The m tiles of l tile [l0, l0 + 32) cover only |m| <= min(L, l0 + 31), so
// small degrees do not run mostly empty tiles.
__device__ __forceinline__ bool ptile_coords(int L, int& n, int& l0, int& mb, int& f)
{
    const int mtiles = (2 * L + 1 + PT - 1) / PT;
    n = (int)blockIdx.x - L;
    l0 = (int)blockIdx.y * PT;
    f = (int)(blockIdx.z / mtiles);
    const int t = (int)(blockIdx.z % mtiles);
    const int mmax = min(L, l0 + PT - 1);
    if (t * PT > 2 * mmax) return false;  // beyond this l tile's m range
    mb = -mmax + t * PT;
    const int an = n < 0 ? -n : n;
    return l0 + PT - 1 >= an && l0 <= L;
}

// group-major pair (g, p) of (m, n) and its group's first degree m0 (consistent with group_pairs)
__device__ __forceinline__ void pair_m0(int m, int n, int& g, int& p, int& m0, int& sign)
{
    pair_of(m, n, g, p);
    m0 = max(abs(m), abs(n));
    const int n0 = g - m0 * m0 - m0;
    sign = ((p == 1 || p == 2) && ((m0 + n0) & 1)) ? -1 : 1;
}

// Per-tile index tables (shared memory): for each m of the tile the
// group-major base (index = base + l), the first degree m0 = max(|m|, |n|)
// (valid l are m0..L) and the pair sign; for each l the packed base
// (index = base + m).  The element loops then do one compare and one address
// add per element.
struct PTileIdx {
    long long gbase[PT];
    int gm0[PT];
    float gsign[PT];
    long long pbase[PT];
};

__device__ __forceinline__ void ptile_index(PTileIdx& t, int L, int n, int l0, int mb, const long long* goff2)
{
    const int B = L + 1;
    if (threadIdx.x < PT) {
        const int m = mb + (int)threadIdx.x;
        if (m < -L || m > L) {
            t.gm0[threadIdx.x] = 0x7fffffff;
            t.gbase[threadIdx.x] = 0;
            t.gsign[threadIdx.x] = 0.f;
        } else {
            int g, pp, m0, sg;
            pair_m0(m, n, g, pp, m0, sg);
            t.gm0[threadIdx.x] = m0;
            t.gbase[threadIdx.x] = goff2[g] + (long long)pp * (B - m0) - m0;
            t.gsign[threadIdx.x] = (float)sg;
        }
    } else if (threadIdx.x < 2 * PT) {
        const int l = l0 + (int)threadIdx.x - PT;
        t.pbase[threadIdx.x - PT] = so3_off(l) + l + (long long)(n + l) * (2 * l + 1);
    }
    __syncthreads();
}

// Functions per CTA of the tiled permutations: the index tables are built once
// and reused, and two functions' tiles are in flight per iteration.
constexpr int PFPC = 8;

// Fg2 (optional): a second group-major array added to Fg on the way (the refinement's correction)
__global__ void __launch_bounds__(256) group_to_packed_tiled(const float2* __restrict__ Fg, float2* __restrict__ F,
                                                             const long long* __restrict__ goff2, int L,
                                                             long long cstride, int batch,
                                                             const float2* __restrict__ Fg2 = nullptr)
{
    __shared__ float2 tile[2][PT][PT + 1];  // [function & 1][m - mb][l - l0]
    __shared__ PTileIdx ix;
    int n, l0, mb, fg;
    if (!ptile_coords(L, n, l0, mb, fg)) return;
    ptile_index(ix, L, n, l0, mb, goff2);
    const int fend = min(batch, (fg + 1) * PFPC);
    for (int f = fg * PFPC; f < fend; f += 2) {
        const int nfn = f + 1 < fend ? 2 : 1;
        // gather: lanes run along l (contiguous in the group-major layout)
#pragma unroll
        for (int u = 0; u < PT * PT / 256; ++u) {
            const int e = threadIdx.x + u * 256;
            const int mi = e / PT, li = e % PT, l = l0 + li;
            if (l < ix.gm0[mi] || l > L) continue;
            const long long o = ix.gbase[mi] + l;
            float2 v0 = Fg[(long long)f * cstride + o], v1 = make_float2(0.f, 0.f);
            if (nfn == 2) v1 = Fg[(long long)(f + 1) * cstride + o];
            if (Fg2) {
                const float2 d0 = Fg2[(long long)f * cstride + o];
                v0 = make_float2(v0.x + d0.x, v0.y + d0.y);
                if (nfn == 2) {
                    const float2 d1 = Fg2[(long long)(f + 1) * cstride + o];
                    v1 = make_float2(v1.x + d1.x, v1.y + d1.y);
                }
            }
            tile[0][mi][li] = v0;
            if (nfn == 2) tile[1][mi][li] = v1;
        }
        __syncthreads();
        // scatter: lanes run along m (contiguous in the packed layout)
#pragma unroll
        for (int u = 0; u < PT * PT / 256; ++u) {
            const int e = threadIdx.x + u * 256;
            const int li = e / PT, mi = e % PT, l = l0 + li;
            if (l < ix.gm0[mi] || l > L) continue;
            const long long o = ix.pbase[li] + mb + mi;
            F[(long long)f * cstride + o] = tile[0][mi][li];
            if (nfn == 2) F[(long long)(f + 1) * cstride + o] = tile[1][mi][li];
        }
        __syncthreads();
    }
}

// packed -> scaled group-major Y = (2l+1) sign F(l, pair)
// raw: the values as they are (the exact contraction scales them itself), else (2l+1) sign F for the GEMM
__global__ void __launch_bounds__(256) packed_to_group_tiled(const float2* __restrict__ F, float2* __restrict__ Y,
                                                             const long long* __restrict__ goff2, int L,
                                                             long long cstride, int batch, bool raw = false)
{
    __shared__ float2 tile[2][PT][PT + 1];  // [function & 1][m - mb][l - l0]
    __shared__ PTileIdx ix;
    int n, l0, mb, fg;
    if (!ptile_coords(L, n, l0, mb, fg)) return;
    ptile_index(ix, L, n, l0, mb, goff2);
    const int fend = min(batch, (fg + 1) * PFPC);
    for (int f = fg * PFPC; f < fend; f += 2) {
        const int nfn = f + 1 < fend ? 2 : 1;
#pragma unroll
        for (int u = 0; u < PT * PT / 256; ++u) {
            const int e = threadIdx.x + u * 256;
            const int li = e / PT, mi = e % PT, l = l0 + li;
            if (l < ix.gm0[mi] || l > L) continue;
            const long long o = ix.pbase[li] + mb + mi;
            tile[0][mi][li] = F[(long long)f * cstride + o];
            if (nfn == 2) tile[1][mi][li] = F[(long long)(f + 1) * cstride + o];
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < PT * PT / 256; ++u) {
            const int e = threadIdx.x + u * 256;
            const int mi = e / PT, li = e % PT, l = l0 + li;
            if (l < ix.gm0[mi] || l > L) continue;
            const float sc = raw ? 1.f : (float)(2 * l + 1) * ix.gsign[mi];
            const long long o = ix.gbase[mi] + l;
            const float2 v0 = tile[0][mi][li];
            Y[(long long)f * cstride + o] = make_float2(sc * v0.x, sc * v0.y);
            if (nfn == 2) {
                const float2 v1 = tile[1][mi][li];
                Y[(long long)(f + 1) * cstride + o] = make_float2(sc * v1.x, sc * v1.y);
            }
        }
        __syncthreads();
    }
}

static dim3 ptile_grid(int L, int batch)
{
    const int mtiles = (2 * L + 1 + PT - 1) / PT;
    const int fgroups = (batch + PFPC - 1) / PFPC;
    return dim3((unsigned)(2 * L + 1), (unsigned)((L + 1 + PT - 1) / PT), (unsigned)(mtiles * fgroups));
}

// S^2: group-major forward output -> packed F(l, m) at l^2 + m + l (one CTA per (l, function)).
__global__ void s2_group_to_packed_kernel(const float2* __restrict__ Fg, float2* __restrict__ F,
                                          const long long* __restrict__ goff2, int L, long long cstride)
{
    const int l = blockIdx.x, f = blockIdx.y;
    const int B = L + 1;
    const float2* src = Fg + (long long)f * cstride;
    float2* dst = F + (long long)f * cstride + (long long)l * l;
    for (int i = threadIdx.x; i < 2 * l + 1; i += blockDim.x) {
        const int m = i - l, g = m < 0 ? -m : m, p = m < 0 ? 1 : 0;
        dst[i] = src[goff2[g] + (long long)p * (B - g) + (l - g)];
    }
}

// S^2: packed F -> group-major Y (pair 0: F(l, m); pair 1: (-1)^m F(l, -m)), one CTA per (m, function).
__global__ void s2_packed_to_group_kernel(const float2* __restrict__ F, float2* __restrict__ Y,
                                          const long long* __restrict__ goff2, int L, long long cstride)
{
    const int m = blockIdx.x, f = blockIdx.y;
    const int nl = L + 1 - m, np = m > 0 ? 2 : 1;
    const float sg = (m & 1) ? -1.f : 1.f;
    const float2* src = F + (long long)f * cstride;
    float2* dst = Y + (long long)f * cstride + goff2[m];
    for (int i = threadIdx.x; i < np * nl; i += blockDim.x) {
        const int p = i / nl, l = m + (i - p * nl);
        const float2 v = src[s2_idx(l, p == 0 ? m : -m)];
        const float sc = p == 0 ? 1.f : sg;
        dst[i] = make_float2(sc * v.x, sc * v.y);
    }
}

// S^2: zero the Nyquist pencil p = B of H'[fn][p][k].
__global__ void s2_zero_nyquist_pencils_kernel(float2* __restrict__ H, int N, long long nf)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf * N) return;
    const long long f = i / N, k = i % N;
    H[f * (long long)N * N + (long long)(N / 2) * N + k] = make_float2(0.f, 0.f);
}

}  // namespace tc

// --------------------------------------------------------------- host side

using namespace tc;

struct TCState {
    int L = 0, B = 0, N = 0, Kp = 0, batch = 0, ntiles = 0, ngroups = 0;
    int csize = 1;                 // CTAs per cluster of the tensor-core GEMM launches (shared table tiles)
    bool refine = false;
    bool real = false;            // real grids (FFTSO3_*_REAL): real samples in, real part out
    bool s2 = false;              // S^2 (Legendre groups g = m, grids N^2) instead of SO(3)
    bool simt = false;            // FP32 CUDA-core beta-sum (FFTSO3_PREC_FP32) instead of tcgen05
    float* d_tab32 = nullptr;     // FP32 table [row][Kp] (simt)
    int lpb[2] = {0, 0};          // generic-N FFT lines per CTA (rows, cols); 0 = heuristic
    int thr[2] = {256, 256};      // generic-N FFT threads per CTA (rows, cols)
    FFTFactors fac;
    const double* d_tw = nullptr;
    float* d_wf = nullptr;
    long long total_rows = 0;
    __nv_bfloat16* d_tab[3] = {nullptr, nullptr, nullptr};
    float2* d_work = nullptr;     // FFT work grid [fn][k][p][q] (two-pass and generic-N FFTs)
    bool fused_fft = false;       // SO(3), N = 64..512: both FFT passes in one launch through an L2 ring
    float2* d_ring = nullptr;     // fused FFT: ring of beta-slice chunks
    size_t ring_elems = 0;
    int* d_fctl = nullptr;        // fused FFT: tile counter and per-chunk completion counts
    float2* d_pencil = nullptr;   // pencils [fn][p][q][k]
    float2* d_resid = nullptr;    // refinement: residual grid (right after d_pencil, in the same allocation)
    float2* d_coef2 = nullptr;    // refinement: correction coefficients
    float2* d_fc = nullptr;       // real kinds: complex coefficients [fn][C]
    long long* d_grow0 = nullptr;
    long long* d_goff2 = nullptr;  // group-major coefficient offsets
    float2* d_fg = nullptr;        // group-major coefficients [fn][C]
    int4* d_items_fwd = nullptr;
    int4* d_items_inv = nullptr;
    int n_items_fwd = 0, n_items_inv = 0;
    std::vector<int4> items_h[2];  // host copies (forward, inverse), for fused launches
    std::vector<int2> iaux_h[2];   // per item (goff2[g], grow0[g]), same order
    std::vector<long long> h_goff2, h_grow0;  // host copies (the launch lists are rebuilt by the cluster tuner)
    int2* d_iaux_fwd = nullptr;
    int2* d_iaux_inv = nullptr;
    int nsm = 0;
    CUtensorMap tmA_fwd[3], tmA_inv[3];
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

bool tc_encode_bf16_2d(CUtensorMap* tm, const void* base, unsigned long long inner, unsigned long long outer,
                       unsigned box_inner, unsigned box_outer)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * 2};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
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
    for (int p = 0; p < 3; ++p)
        if (s->d_tab[p]) cudaFree(s->d_tab[p]);
    void* ptrs[] = {s->d_tab32, s->d_wf, s->d_work, s->d_ring, s->d_fctl, s->d_pencil, s->d_coef2, s->d_fc, s->d_grow0, s->d_goff2, s->d_fg,
                    s->d_items_fwd, s->d_items_inv, s->d_iaux_fwd, s->d_iaux_inv, s->d_err};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    delete s;
}

long long tc_device_bytes(const TCState* s) { return s ? s->bytes : 0; }

static int autotune_fft(TCState* s, std::string& err);
static int autotune_cluster(TCState* s, std::string& err);
static int launch_gemm(TCState* s, bool fwd, cudaStream_t st, std::string& err, float2* cout = nullptr,
                       int terms = 3);
static long long coeffs_per_fn(const TCState* s);
static long long grid_per_fn(const TCState* s);

// The tensor-core GEMM's launch lists for clusters of `csize` CTAs (a power of two <= column tiles): with
// csize > 1, blocks of csize items (same group and row tile, consecutive column tiles; tiles past the batch
// are empty) go to one cluster, which reads each table tile once for the block; csize = 1 takes the one-CTA
// lists.  Replaces the device lists and sets s->csize.
static int set_launch_lists(TCState* s, int csize, std::string& err)
{
    const int N = s->N;
    std::vector<int4> itf, iti;
    if (csize <= 1) {
        itf = s->items_h[0];
        iti = s->items_h[1];
        csize = 1;
    } else {
        const int CLs = csize, ntb = (s->ntiles + CLs - 1) / CLs;
        std::vector<std::vector<int4>> blocks;
        for (int g = 0; g < s->ngroups; ++g) {
            int m0 = g, n0 = 0;
            if (!s->s2) group_mn(g, m0, n0);
            const int nl = s->B - m0;
            for (int mt = 0; mt * BM < nl; ++mt)
                for (int b = 0; b < ntb; ++b)
                    for (int r = 0; r < CLs; ++r) itf.push_back(make_int4(g, mt, b * CLs + r, item_w(m0, n0)));
            for (int mt = 0; mt * BM < N; ++mt)
                for (int b = 0; b < ntb; ++b) {
                    std::vector<int4> blk;
                    for (int r = 0; r < CLs; ++r) blk.push_back(make_int4(g, mt, b * CLs + r, item_w(m0, n0)));
                    blocks.push_back(blk);
                }
        }
        std::stable_sort(blocks.begin(), blocks.end(), [&](const std::vector<int4>& a, const std::vector<int4>& b) {
            const int ma = a[0].w >> 16, mb = b[0].w >> 16;
            return (s->B - ma + BK - 1) / BK > (s->B - mb + BK - 1) / BK;
        });
        for (const auto& blk : blocks) iti.insert(iti.end(), blk.begin(), blk.end());
    }
    std::vector<int2> auxf(itf.size()), auxi(iti.size());
    for (size_t i = 0; i < itf.size(); ++i)
        auxf[i] = make_int2((int)s->h_goff2[itf[i].x], (int)s->h_grow0[itf[i].x]);
    for (size_t i = 0; i < iti.size(); ++i)
        auxi[i] = make_int2((int)s->h_goff2[iti[i].x], (int)s->h_grow0[iti[i].x]);
    // replace the device lists
    auto drop = [&](void* p, size_t bytes) {
        if (p) {
            cudaFree(p);
            s->bytes -= (long long)bytes;
        }
    };
    drop(s->d_items_fwd, sizeof(int4) * (size_t)s->n_items_fwd);
    drop(s->d_items_inv, sizeof(int4) * (size_t)s->n_items_inv);
    drop(s->d_iaux_fwd, sizeof(int2) * (size_t)s->n_items_fwd);
    drop(s->d_iaux_inv, sizeof(int2) * (size_t)s->n_items_inv);
    s->d_items_fwd = s->d_items_inv = nullptr;
    s->d_iaux_fwd = s->d_iaux_inv = nullptr;
    s->n_items_fwd = s->n_items_inv = 0;
    int rc;
    if ((rc = tc_alloc(s, (void**)&s->d_items_fwd, sizeof(int4) * itf.size(), err))) return rc;
    s->n_items_fwd = (int)itf.size();
    if ((rc = tc_alloc(s, (void**)&s->d_iaux_fwd, sizeof(int2) * itf.size(), err))) return rc;
    if ((rc = tc_alloc(s, (void**)&s->d_items_inv, sizeof(int4) * iti.size(), err))) return rc;
    s->n_items_inv = (int)iti.size();
    if ((rc = tc_alloc(s, (void**)&s->d_iaux_inv, sizeof(int2) * iti.size(), err))) return rc;
    cudaMemcpy(s->d_items_fwd, itf.data(), sizeof(int4) * itf.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(s->d_items_inv, iti.data(), sizeof(int4) * iti.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(s->d_iaux_fwd, auxf.data(), sizeof(int2) * itf.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(s->d_iaux_inv, auxi.data(), sizeof(int2) * iti.size(), cudaMemcpyHostToDevice);
    s->csize = csize;
    return FFTSO3_SUCCESS;
}

int tc_create(TCState** out, int L, int N, int batch, const double* d_table_fp64, const std::vector<long long>& goff,
              long long table_elems, const double* d_tw, const double* d_w, bool refine, bool real, bool s2,
              bool autotune, bool simt, std::string& err)
{
    *out = nullptr;
    if (N > MAXN) {
        err = "tensor-core path supports 2(l_max+1) <= 1024";
        return FFTSO3_ERR_UNSUPPORTED;
    }
    TCState* s = new TCState();
    s->L = L;
    s->B = L + 1;
    s->N = N;
    s->Kp = (N + 63) / 64 * 64;
    s->batch = batch;
    s->s2 = s2;
    s->simt = simt;
    // grid limits: the coefficient permutations run ceil((2L+1)/32) m tiles x ceil(batch / 8) function groups in
    // gridDim.z, the per-function conversions take the batch in gridDim.y
    if (batch > 65535 || (!s2 && (long long)((2 * L + 1 + 31) / 32) * ((batch + PFPC - 1) / PFPC) > 65535)) {
        err = "batch too large for this l_max (at most 65535 functions, and 65535 / ceil((2 l_max + 1) / 32) "
              "groups of 8 functions for SO(3))";
        delete s;
        return FFTSO3_ERR_UNSUPPORTED;
    }
    s->ntiles = s2 ? (batch + FPT_S2 - 1) / FPT_S2 : (batch + FPT - 1) / FPT;
    s->ngroups = s2 ? s->B : s->B * s->B;
    s->refine = refine;
    s->real = real;
    make_fft_factors_prime_first(N, s->fac);
    s->d_tw = d_tw;
    s->total_rows = table_elems / N;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, dev);
    int rc;
    auto bail = [&](int code) {
        tc_destroy(s);
        return code;
    };
    // FP32 weights
    {
        std::vector<double> w(N);
        cudaMemcpy(w.data(), d_w, sizeof(double) * N, cudaMemcpyDeviceToHost);
        std::vector<float> wf(N);
        for (int k = 0; k < N; ++k) wf[k] = (float)w[k];
        if ((rc = tc_alloc(s, (void**)&s->d_wf, sizeof(float) * N, err))) return bail(rc);
        cudaMemcpy(s->d_wf, wf.data(), sizeof(float) * N, cudaMemcpyHostToDevice);
    }
    // table: three BF16 planes (tensor cores) or one FP32 copy (CUDA cores)
    const long long tot = s->total_rows * s->Kp;
    if (simt) {
        if ((rc = tc_alloc(s, (void**)&s->d_tab32, sizeof(float) * tot, err))) return bail(rc);
        table_fp32_kernel<<<(unsigned)((tot + 255) / 256), 256>>>(d_table_fp64, s->d_tab32, s->total_rows, N, s->Kp);
    } else {
        for (int p = 0; p < 3; ++p)
            if ((rc = tc_alloc(s, (void**)&s->d_tab[p], sizeof(__nv_bfloat16) * tot, err))) return bail(rc);
        table_split_kernel<<<(unsigned)((tot + 255) / 256), 256>>>(d_table_fp64, s->d_tab[0], s->d_tab[1],
                                                                   s->d_tab[2], s->total_rows, N, s->Kp);
    }
    {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            err = std::string("table split: ") + cudaGetErrorString(e);
            return bail(FFTSO3_ERR_CUDA);
        }
    }
    const size_t gridel = (size_t)batch * N * N * (s2 ? 1 : N);
    const long long C = s2 ? (long long)s->B * s->B : so3_off(s->B);
    // FFT scratch: the fused two-pass FFT needs only a ring of beta-slice chunks
    // (FFTSO3_TWO_PASS_FFT=1 in the environment selects the two-launch form, for comparison)
    {
        const char* ev = getenv("FFTSO3_TWO_PASS_FFT");
        s->fused_fft = !s2 && fft_grid_fused_supported(N) && !(ev && ev[0] == '1');
    }
    if (s->fused_fft) {
        s->ring_elems = fft_grid_fused_ring_elems(N);
        if ((rc = tc_alloc(s, (void**)&s->d_ring, sizeof(float2) * s->ring_elems, err))) return bail(rc);
        if ((rc = tc_alloc(s, (void**)&s->d_fctl, sizeof(int) * fft_grid_fused_ctl_ints(batch, N), err)))
            return bail(rc);
    } else if (!(s2 && fft_fast_supported(N))) {
        if ((rc = tc_alloc(s, (void**)&s->d_work, sizeof(float2) * gridel, err))) return bail(rc);
    }
    // refinement: the residual buffer follows the pencils in one allocation, so that together they hold one
    // 16-byte (double-float) element per pencil place for the exact inverse
    if ((rc = tc_alloc(s, (void**)&s->d_pencil, sizeof(float2) * gridel * (refine ? 2 : 1), err))) return bail(rc);
    if (real)
        if ((rc = tc_alloc(s, (void**)&s->d_fc, sizeof(float2) * (size_t)batch * C, err))) return bail(rc);
    if (refine) {
        s->d_resid = s->d_pencil + gridel;
        if ((rc = tc_alloc(s, (void**)&s->d_coef2, sizeof(float2) * (size_t)batch * C, err))) return bail(rc);
    }
    // group rows and work items; the inverse list is ordered by decreasing cost
    std::vector<long long> grow0(s->ngroups), goff2(s->ngroups + 1);
    std::vector<int4> itf, iti;
    long long acc2 = 0;
    for (int g = 0; g < s->ngroups; ++g) {
        int m0 = g, n0 = 0;
        if (!s2) group_mn(g, m0, n0);
        grow0[g] = goff[g] / N;
        const int nl = s->B - m0;
        goff2[g] = acc2;
        acc2 += (long long)(s2 ? (m0 > 0 ? 2 : 1) : group_pairs(m0, n0).np) * nl;
        for (int nt = 0; nt < s->ntiles; ++nt) {
            for (int mt = 0; mt * BM < nl; ++mt) itf.push_back(make_int4(g, mt, nt, item_w(m0, n0)));
            for (int mt = 0; mt * BM < N; ++mt) iti.push_back(make_int4(g, mt, nt, item_w(m0, n0)));
        }
    }
    std::stable_sort(iti.begin(), iti.end(), [&](const int4& a, const int4& b) {
        const int ma = a.w >> 16, mb = b.w >> 16;
        return (s->B - ma + BK - 1) / BK > (s->B - mb + BK - 1) / BK;
    });
    s->items_h[0] = itf;  // one-CTA order, for fused launches over several plans
    s->items_h[1] = iti;
    // launch lists: clusters of C CTAs (C a power of two <= column tiles, at most FFTSO3_GEMM_CLUSTER, default
    // 2) share each table tile; FFTSO3_FLAG_AUTOTUNE times C = 1, 2, 4 (below)
    int csize0 = 1;
    {
        const char* ev = getenv("FFTSO3_GEMM_CLUSTER");
        int cmax = ev ? atoi(ev) : 2;
        cmax = cmax >= 4 ? 4 : cmax >= 2 ? 2 : 1;
        if (!simt)
            while (csize0 * 2 <= cmax && csize0 * 2 <= s->ntiles) csize0 *= 2;
    }
    goff2[s->ngroups] = acc2;
    if (acc2 != C) {
        err = "internal: group-major layout does not cover the coefficients";
        return bail(FFTSO3_ERR_CUDA);
    }
    if (acc2 > 0x7fffffffLL || s->total_rows > 0x7fffffffLL) {
        err = "internal: per-item offsets exceed 32 bits";
        return bail(FFTSO3_ERR_UNSUPPORTED);
    }
    for (int d = 0; d < 2; ++d) {
        s->iaux_h[d].resize(s->items_h[d].size());
        for (size_t i = 0; i < s->items_h[d].size(); ++i) {
            const int g = s->items_h[d][i].x;
            s->iaux_h[d][i] = make_int2((int)goff2[g], (int)grow0[g]);
        }
    }
    s->h_goff2 = goff2;
    s->h_grow0 = grow0;
    if ((rc = tc_alloc(s, (void**)&s->d_grow0, sizeof(long long) * grow0.size(), err))) return bail(rc);
    if ((rc = tc_alloc(s, (void**)&s->d_goff2, sizeof(long long) * goff2.size(), err))) return bail(rc);
    if ((rc = tc_alloc(s, (void**)&s->d_fg, sizeof(float2) * (size_t)batch * acc2, err))) return bail(rc);
    cudaMemcpy(s->d_goff2, goff2.data(), sizeof(long long) * goff2.size(), cudaMemcpyHostToDevice);
    if ((rc = set_launch_lists(s, csize0, err))) return bail(rc);
    if ((rc = tc_alloc(s, (void**)&s->d_err, sizeof(int), err))) return bail(rc);
    cudaMemcpy(s->d_grow0, grow0.data(), sizeof(long long) * grow0.size(), cudaMemcpyHostToDevice);
    cudaMemset(s->d_err, 0, sizeof(int));
    for (int p = 0; p < 3 && !simt; ++p) {
        bool ok = tc_encode_bf16_2d(&s->tmA_fwd[p], s->d_tab[p], s->Kp, s->total_rows, 64, BM) &&
                  tc_encode_bf16_2d(&s->tmA_inv[p], s->d_tab[p], s->Kp, s->total_rows, 64, BK);
        if (!ok) {
            err = "cuTensorMapEncodeTiled failed";
            return bail(FFTSO3_ERR_CUDA);
        }
    }
    cudaError_t e = cudaSuccess;
    const void* kernels[9] = {
        (const void*)so3_tc_gemm_kernel<true, false, false>, (const void*)so3_tc_gemm_kernel<false, false, false>,
        (const void*)so3_tc_gemm_kernel<true, true, false>,  (const void*)so3_tc_gemm_kernel<false, true, false>,
        (const void*)so3_tc_gemm_kernel<true, false, true>,  (const void*)so3_tc_gemm_kernel<false, false, true>,
        (const void*)so3_tc_gemm_kernel<true, true, true>,   (const void*)so3_tc_gemm_kernel<false, true, true>,
        (const void*)so3_tc_gemm_kernel<true, false, false, 1>};
    for (int i = 0; i < 9 && e == cudaSuccess; ++i)
        e = cudaFuncSetAttribute(kernels[i], cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) {
        err = std::string("tensor-core kernel attributes: ") + cudaGetErrorString(e);
        return bail(FFTSO3_ERR_CUDA);
    }
    if (autotune && !fft_fast_supported(N))
        if ((rc = autotune_fft(s, err))) return bail(rc);
    if (autotune && !simt && s->ntiles > 1)
        if ((rc = autotune_cluster(s, err))) return bail(rc);
    *out = s;
    return FFTSO3_SUCCESS;
}

static FFTLaunch fft_launch(const TCState* s, const void* in, void* out, bool cols, bool real_in = false,
                            bool real_out = false)
{
    FFTLaunch L;
    const int N = s->N;
    L.in = in;
    L.out = out;
    L.fac = s->fac;
    L.tw = s->d_tw;
    L.fp64 = false;
    L.real_in = real_in;
    L.real_out = real_out;
    L.nlines = (long long)s->batch * N * (s->s2 ? 1 : N);
    // lines per CTA: about 2048 elements per CTA (small N would otherwise leave most threads idle)
    int lpb = 1;
    while (lpb < 256 && (lpb * 2) * N <= 2048 && fft_smem_bytes(N, lpb * 2, false) <= 100 * 1024) lpb *= 2;
    L.threads = s->thr[cols ? 1 : 0];
    if (!cols) {
        L.lpb = s->lpb[0] ? s->lpb[0] : lpb;
        L.inner = 1;
        L.ostride = N;
        L.istride = 0;
        L.es = 1;
        L.lines_fastest = false;
    } else {
        L.lpb = lpb < 16 ? 16 : lpb;  // >= 16 adjacent lines: 128-byte segments
        while (L.lpb > 1 && fft_smem_bytes(N, L.lpb, false) > 100 * 1024) L.lpb /= 2;
        if (s->lpb[1]) L.lpb = s->lpb[1];
        L.inner = N;
        L.ostride = (long long)N * N;
        L.istride = 1;
        L.es = N;
        L.lines_fastest = true;
    }
    return L;
}

// ---- autotuner of the generic-N FFT launch shape (lines per CTA, threads per CTA)
//
// For N that the register FFT does not cover, the best lines-per-CTA and CTA
// size depend on N (its factors, the shared memory per line) and on the pass
// (rows: lines contiguous; columns: lines adjacent).  With FFTSO3_FLAG_AUTOTUNE
// the plan times every candidate on its own workspace (about 32 M samples,
// one warm-up and three timed launches each, CUDA events) and keeps the
// fastest; choices are cached per (N, pass, real input/output) for the process,
// so the many plans of an uneven batch tune each N once.
struct TuneKey {
    int N, cols, real_in, real_out;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(N, cols, real_in, real_out) < std::tie(o.N, o.cols, o.real_in, o.real_out);
    }
};
static std::mutex g_tune_mutex;
static std::map<TuneKey, std::pair<int, int>> g_tune_cache;

static int autotune_fft(TCState* s, std::string& err)
{
    const int N = s->N;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        err = "autotune: cudaStreamCreate";
        return FFTSO3_ERR_CUDA;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const size_t gridel = (size_t)s->batch * N * N * (s->s2 ? 1 : N);
    cudaMemsetAsync(s->d_work, 0, sizeof(float2) * gridel, st);
    cudaMemsetAsync(s->d_pencil, 0, sizeof(float2) * gridel, st);
    const int npass = s->s2 ? 1 : 2;
    int rc = FFTSO3_SUCCESS;
    for (int cols = 0; cols < npass && rc == FFTSO3_SUCCESS; ++cols) {
        const TuneKey key{N, cols, (!cols && s->real) ? 1 : 0, 0};
        {
            std::lock_guard<std::mutex> lk(g_tune_mutex);
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) {
                s->lpb[cols] = it->second.first;
                s->thr[cols] = it->second.second;
                continue;
            }
        }
        float best = 1e30f;
        int blpb = 0, bthr = 256;
        for (int thr = 128; thr <= 256; thr *= 2) {
            for (int lpb = cols ? 4 : 1; lpb <= 256; lpb *= 2) {
                if ((long long)lpb * N > 8192 || fft_smem_bytes(N, lpb, false) > 100 * 1024) break;
                s->lpb[cols] = lpb;
                s->thr[cols] = thr;
                FFTLaunch L = fft_launch(s, s->d_pencil, s->d_work, cols != 0, key.real_in != 0, false);
                L.nlines = std::min<long long>(L.nlines, (32LL << 20) / N / lpb * lpb + lpb);
                if (launch_fft_lines(L, st) != cudaSuccess) continue;
                cudaEventRecord(e0, st);
                for (int r = 0; r < 3; ++r) launch_fft_lines(L, st);
                cudaEventRecord(e1, st);
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    err = std::string("autotune: ") + cudaGetErrorString(cudaGetLastError());
                    rc = FFTSO3_ERR_CUDA;
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best) {
                    best = ms;
                    blpb = lpb;
                    bthr = thr;
                }
            }
        }
        s->lpb[cols] = blpb;
        s->thr[cols] = bthr;
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        g_tune_cache[key] = {blpb, bthr};
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    return rc;
}

// FFTSO3_FLAG_AUTOTUNE: the GEMM's cluster size (1, 2 or 4 CTAs sharing each table tile, at most the column
// tiles), timed on the plan's own buffers (one warm-up, then two forward and two inverse GEMMs each, CUDA
// events; the buffers' contents do not matter to the timing and are overwritten by every call), cached per
// (l_max, batch, family) for the process.
static std::map<std::tuple<int, int, bool>, int> g_cluster_cache;

static int autotune_cluster(TCState* s, std::string& err)
{
    const auto key = std::make_tuple(s->L, s->batch, s->s2);
    {
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        auto it = g_cluster_cache.find(key);
        if (it != g_cluster_cache.end()) return it->second == s->csize ? FFTSO3_SUCCESS : set_launch_lists(s, it->second, err);
    }
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        err = "autotune: cudaStreamCreate";
        return FFTSO3_ERR_CUDA;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemsetAsync(s->d_pencil, 0, sizeof(float2) * (size_t)s->batch * grid_per_fn(s), st);
    cudaMemsetAsync(s->d_fg, 0, sizeof(float2) * (size_t)s->batch * coeffs_per_fn(s), st);
    const int first = s->csize;
    float best = 1e30f;
    int bestc = first, rc = FFTSO3_SUCCESS;
    for (int c = 1; c <= 4 && c <= s->ntiles && rc == FFTSO3_SUCCESS; c *= 2) {
        if ((rc = set_launch_lists(s, c, err))) break;
        if ((rc = launch_gemm(s, true, st, err)) || (rc = launch_gemm(s, false, st, err))) {
            if (rc == FFTSO3_ERR_UNSUPPORTED) {  // no cluster of c CTAs fits: not a candidate
                rc = FFTSO3_SUCCESS;
                cudaGetLastError();
                continue;
            }
            break;
        }
        cudaEventRecord(e0, st);
        for (int r = 0; r < 2 && rc == FFTSO3_SUCCESS; ++r)
            if ((rc = launch_gemm(s, true, st, err)) == FFTSO3_SUCCESS) rc = launch_gemm(s, false, st, err);
        cudaEventRecord(e1, st);
        if (rc) break;
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            err = std::string("autotune: ") + cudaGetErrorString(cudaGetLastError());
            rc = FFTSO3_ERR_CUDA;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            bestc = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (tc_status(s) != 0) {
        err = "autotune: the tensor-core GEMM gave up a bounded wait";
        return FFTSO3_ERR_CUDA;
    }
    {
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        g_cluster_cache[key] = bestc;
    }
    return set_launch_lists(s, bestc, err);
}

#define TCK(call)                                                          \
    do {                                                                   \
        cudaError_t _e = (call);                                           \
        if (_e != cudaSuccess) {                                           \
            err = std::string(#call) + ": " + cudaGetErrorString(_e);      \
            return FFTSO3_ERR_CUDA;                                        \
        }                                                                  \
    } while (0)

static GemmArgs gemm_args(const TCState* s)
{
    GemmArgs a;
    a.items = nullptr;
    a.iaux = nullptr;
    a.nitems = 0;
    a.csize = 1;
    a.grow0 = s->d_grow0;
    a.goff2 = s->d_goff2;
    a.L = s->L;
    a.N = s->N;
    a.Kp = s->Kp;
    a.batch = s->batch;
    a.fstride = (long long)s->N * s->N * (s->s2 ? 1 : s->N);
    a.cstride = s->s2 ? (long long)s->B * s->B : so3_off(s->B);
    a.pin = nullptr;
    a.cin = nullptr;
    a.cout = nullptr;
    a.pout = nullptr;
    a.wf = s->d_wf;
    a.err = s->d_err;
    return a;
}

// cout: the forward's group-major output (default: the plan's d_fg); terms: 1 selects the one-term kernel (SO(3)
// forward only)
static int launch_gemm(TCState* s, bool fwd, cudaStream_t st, std::string& err, float2* cout, int terms)
{
    GemmArgs a = gemm_args(s);
    a.items = fwd ? s->d_items_fwd : s->d_items_inv;
    a.iaux = fwd ? s->d_iaux_fwd : s->d_iaux_inv;
    a.nitems = fwd ? s->n_items_fwd : s->n_items_inv;
    if (fwd) {
        a.pin = s->d_pencil;
        a.cout = cout ? cout : s->d_fg;
    } else {
        a.cin = s->d_fg;
        a.pout = s->d_pencil;
    }
    if (s->simt) {
        if (fwd && s->s2)
            so3_fp32_gemm_kernel<true, true><<<a.nitems, 256, 0, st>>>(s->d_tab32, a);
        else if (fwd)
            so3_fp32_gemm_kernel<true, false><<<a.nitems, 256, 0, st>>>(s->d_tab32, a);
        else if (s->s2)
            so3_fp32_gemm_kernel<false, true><<<a.nitems, 256, 0, st>>>(s->d_tab32, a);
        else
            so3_fp32_gemm_kernel<false, false><<<a.nitems, 256, 0, st>>>(s->d_tab32, a);
        TCK(cudaGetLastError());
        return FFTSO3_SUCCESS;
    }
    const CUtensorMap* tm = fwd ? s->tmA_fwd : s->tmA_inv;
    auto kern = fwd ? (s->s2 ? so3_tc_gemm_kernel<true, true, false>
                             : (terms == 1 ? so3_tc_gemm_kernel<true, false, false, 1>
                                           : so3_tc_gemm_kernel<true, false, false>))
                    : (s->s2 ? so3_tc_gemm_kernel<false, true, false> : so3_tc_gemm_kernel<false, false, false>);
    if (s->csize == 1) {
        const int nctas = a.nitems < s->nsm ? a.nitems : s->nsm;
        kern<<<nctas, THREADS, SMEM_BYTES, st>>>(tm[0], tm[1], tm[2], a, nullptr);
        TCK(cudaGetLastError());
        return FFTSO3_SUCCESS;
    }
    // clusters of csize CTAs (the item list is in blocks of csize): as many clusters as fit at once
    a.csize = s->csize;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)s->csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = SMEM_BYTES;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3((unsigned)s->csize);
    int nclusters = 0;
    TCK(cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg));
    if (nclusters < 1) {
        err = "tensor-core GEMM: no cluster of " + std::to_string(s->csize) + " CTAs fits on this device";
        return FFTSO3_ERR_UNSUPPORTED;
    }
    long long nctas = (long long)nclusters * s->csize;
    if (nctas > a.nitems) nctas = a.nitems;  // a.nitems is a multiple of csize
    cfg.gridDim = dim3((unsigned)nctas);
    TCK(cudaLaunchKernelEx(&cfg, kern, tm[0], tm[1], tm[2], a, (const GemmSeg*)nullptr));
    return FFTSO3_SUCCESS;
}

static long long coeffs_per_fn(const TCState* s) { return s->s2 ? (long long)s->B * s->B : so3_off(s->B); }
static long long grid_per_fn(const TCState* s) { return (long long)s->N * s->N * (s->s2 ? 1 : s->N); }

// grid -> k-contiguous pencils (SO(3): [fn][p][q][k], S^2: [fn][p][k]); grid is
// float2, or float when s->real.
static int fft_forward(TCState* s, const void* grid, cudaStream_t st, StageTimer* T, std::string& err)
{
    const long long N = s->N;
    if (fft_fast_supported(s->N)) {
        // register-resident FFTs; the last pass writes the k-contiguous pencils directly
        if (s->fused_fft) {
            T->begin(ST_FFT_2D, st);
            TCK(launch_fft_grid_fused(grid, s->d_pencil, s->d_ring, s->ring_elems, s->d_fctl, s->d_err, s->batch, s->N, 1, s->d_tw,
                                      st, s->real));
            T->end(st);
            return FFTSO3_SUCCESS;
        }
        T->begin(ST_FFT_ROWS, st);
        if (s->s2)
            TCK(launch_fft_s2_pass(grid, s->d_pencil, s->batch, s->N, 1, s->d_tw, st, s->real));
        else
            TCK(launch_fft_grid_pass(grid, s->d_work, s->batch, s->N, 1, s->d_tw, st, s->real));
        T->end(st);
        if (!s->s2) {
            T->begin(ST_FFT_COLS, st);
            TCK(launch_fft_grid_pass(s->d_work, s->d_pencil, s->batch, s->N, 2, s->d_tw, st));
            T->end(st);
        }
        return FFTSO3_SUCCESS;
    }
    T->begin(ST_FFT_ROWS, st);
    TCK(launch_fft_lines(fft_launch(s, grid, s->d_work, false, s->real, false), st));
    T->end(st);
    if (!s->s2) {
        T->begin(ST_FFT_COLS, st);
        TCK(launch_fft_lines(fft_launch(s, s->d_work, s->d_work, true), st));
        T->end(st);
    }
    T->begin(ST_PACK_FWD, st);
    const long long Cc = s->s2 ? N : N * N;  // [k][rest] -> [rest][k]
    dim3 tg((unsigned)((Cc + 31) / 32), (unsigned)((N + 31) / 32), (unsigned)s->batch);
    transpose_kernel<<<tg, dim3(32, 8), 0, st>>>(s->d_work, s->d_pencil, N, Cc);
    TCK(cudaGetLastError());
    T->end(st);
    return FFTSO3_SUCCESS;
}

// k-contiguous pencils -> grid (float2, or the real parts when s->real).
static int fft_inverse(TCState* s, void* grid, cudaStream_t st, StageTimer* T, std::string& err)
{
    const long long N = s->N;
    if (fft_fast_supported(s->N)) {
        if (s->s2) {
            T->begin(ST_FFT_ROWS, st);
            TCK(launch_fft_s2_pass(s->d_pencil, grid, s->batch, s->N, -1, s->d_tw, st, s->real));
            T->end(st);
            return FFTSO3_SUCCESS;
        }
        if (s->fused_fft) {
            T->begin(ST_FFT_2D, st);
            TCK(launch_fft_grid_fused(s->d_pencil, grid, s->d_ring, s->ring_elems, s->d_fctl, s->d_err, s->batch, s->N, -1, s->d_tw,
                                      st, s->real));
            T->end(st);
            return FFTSO3_SUCCESS;
        }
        T->begin(ST_FFT_COLS, st);
        TCK(launch_fft_grid_pass(s->d_pencil, s->d_work, s->batch, s->N, -2, s->d_tw, st));
        T->end(st);
        T->begin(ST_FFT_ROWS, st);
        TCK(launch_fft_grid_pass(s->d_work, grid, s->batch, s->N, -1, s->d_tw, st, s->real));
        T->end(st);
        return FFTSO3_SUCCESS;
    }
    T->begin(ST_PACK_INV, st);
    {
        const long long Cc = s->s2 ? N : N * N;
        dim3 tg((unsigned)((N + 31) / 32), (unsigned)((Cc + 31) / 32), (unsigned)s->batch);
        transpose_kernel<<<tg, dim3(32, 8), 0, st>>>(s->d_pencil, s->d_work, Cc, N);
        TCK(cudaGetLastError());
    }
    T->end(st);
    if (s->s2) {
        T->begin(ST_FFT_ROWS, st);
        TCK(launch_fft_lines(fft_launch(s, s->d_work, grid, false, false, s->real), st));
        T->end(st);
        return FFTSO3_SUCCESS;
    }
    T->begin(ST_FFT_ROWS, st);
    TCK(launch_fft_lines(fft_launch(s, s->d_work, s->d_work, false), st));
    T->end(st);
    T->begin(ST_FFT_COLS, st);
    TCK(launch_fft_lines(fft_launch(s, s->d_work, grid, true, false, s->real), st));
    T->end(st);
    return FFTSO3_SUCCESS;
}

// real_out (S^2 real kinds): write the real coefficients straight from the GEMM output instead of F.
static int tc_forward_once(TCState* s, const void* grid, float2* F, cudaStream_t st, StageTimer* T,
                           std::string& err, void* real_out = nullptr)
{
    int rc = fft_forward(s, grid, st, T, err);
    if (rc) return rc;
    T->begin(ST_GEMM_FWD, st);
    if ((rc = launch_gemm(s, true, st, err))) return rc;
    T->end(st);
    T->begin(ST_BASIS, st);
    if (real_out)
        TCK(launch_s2_group_to_real(s->d_fg, real_out, s->d_goff2, s->L, s->batch, st));
    else if (s->s2)
        s2_group_to_packed_kernel<<<dim3(s->B, s->batch), 256, 0, st>>>(s->d_fg, F, s->d_goff2, s->L,
                                                                       coeffs_per_fn(s));
    else
        group_to_packed_tiled<<<ptile_grid(s->L, s->batch), 256, 0, st>>>(s->d_fg, F, s->d_goff2, s->L,
                                                                    coeffs_per_fn(s), s->batch);
    TCK(cudaGetLastError());
    T->end(st);
    return FFTSO3_SUCCESS;
}

// real_in (S^2 real kinds): read the real coefficients straight into the GEMM input instead of F.
static int tc_inverse_once(TCState* s, const float2* F, void* grid, cudaStream_t st, StageTimer* T,
                           std::string& err, const void* real_in = nullptr)
{
    const long long N = s->N;
    T->begin(ST_NYQUIST, st);
    if (s->s2) {
        const long long tot = (long long)s->batch * N;
        s2_zero_nyquist_pencils_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(s->d_pencil, (int)N, s->batch);
    } else {
        const long long tot = (long long)s->batch * 2 * N * N;
        zero_nyquist_pencils_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(s->d_pencil, (int)N, s->batch);
    }
    TCK(cudaGetLastError());
    T->end(st);
    T->begin(ST_BASIS, st);
    if (real_in)
        TCK(launch_s2_real_to_group(real_in, s->d_fg, s->d_goff2, s->L, s->batch, st));
    else if (s->s2)
        s2_packed_to_group_kernel<<<dim3(s->ngroups, s->batch), 128, 0, st>>>(F, s->d_fg, s->d_goff2, s->L,
                                                                             coeffs_per_fn(s));
    else
        packed_to_group_tiled<<<ptile_grid(s->L, s->batch), 256, 0, st>>>(F, s->d_fg, s->d_goff2, s->L,
                                                                          coeffs_per_fn(s), s->batch);
    TCK(cudaGetLastError());
    T->end(st);
    T->begin(ST_GEMM_INV, st);
    int rc = launch_gemm(s, false, st, err);
    if (rc) return rc;
    T->end(st);
    return fft_inverse(s, grid, st, T, err);
}

int tc_forward(TCState* s, const void* grid, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    // real kinds: complex coefficients in d_fc, then the real basis
    // (fdcl_FFTSO3.cpp:1169-1181, fdcl_FFTS2.cpp:424-436); the S^2 real kinds
    // write the real coefficients straight from the GEMM output
    if (s->real && s->s2) return tc_forward_once(s, grid, nullptr, st, T, err, coeffs);
    float2* Fc = s->real ? s->d_fc : (float2*)coeffs;
    int rc = tc_forward_once(s, grid, Fc, st, T, err);
    if (rc) return rc;
    if (s->real) {
        T->begin(ST_BASIS, st);
        if (s->s2)
            TCK(launch_s2_c2r(Fc, coeffs, false, s->L, s->batch, st));
        else
            TCK(launch_so3_c2r(Fc, coeffs, false, s->L, s->batch, st));
        T->end(st);
    }
    return FFTSO3_SUCCESS;
}

void* tc_resid_buffer(TCState* s) { return s ? (void*)s->d_resid : nullptr; }

float2* tc_pencil_buffer(TCState* s) { return s ? s->d_pencil : nullptr; }

void* tc_exact_buffer(TCState* s) { return s && s->d_resid ? (void*)s->d_pencil : nullptr; }

const float2* tc_group_from_packed(TCState* s, const void* packed, int f0, int nb, cudaStream_t st)
{
    const long long C = coeffs_per_fn(s);
    float2* out = s->d_fg + (long long)f0 * C;
    packed_to_group_tiled<<<ptile_grid(s->L, nb), 256, 0, st>>>((const float2*)packed + (long long)f0 * C, out,
                                                                 s->d_goff2, s->L, C, nb, true);
    return cudaGetLastError() == cudaSuccess ? out : nullptr;
}

// forward from pencils already in d_pencil: GEMM (terms: see launch_gemm), then the packed (and real-basis)
// coefficients
static int forward_from_pencils(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err,
                                int terms = 3)
{
    T->begin(ST_GEMM_FWD, st);
    int rc = launch_gemm(s, true, st, err, nullptr, terms);
    if (rc) return rc;
    T->end(st);
    return tc_forward_finish(s, coeffs, st, T, err);
}

int tc_forward_pencils(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    if (s->s2) {
        err = "internal: pencil-domain forward is SO(3) only";
        return FFTSO3_ERR_CUDA;
    }
    return forward_from_pencils(s, coeffs, st, T, err);
}

float2* tc_group_buffer(TCState* s) { return s ? s->d_fg : nullptr; }

int tc_gemm_forward_group(TCState* s, cudaStream_t st, StageTimer* T, std::string& err)
{
    T->begin(ST_GEMM_FWD, st);
    int rc = launch_gemm(s, true, st, err);
    if (rc) return rc;
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_refine_finish_group(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    if (!s->refine || !s->d_coef2 || s->s2 || s->real) {
        err = "internal: group-major refinement is for complex SO(3) refined plans";
        return FFTSO3_ERR_CUDA;
    }
    // the correction's GEMM into d_coef2 (group-major), then one permutation that adds it to F0 (d_fg).  One BF16
    // term: the residual is ~5e-7 of the samples' spectrum, so the term's 2^-9 relative rounding leaves ~1e-9.
    T->begin(ST_GEMM_FWD, st);
    int rc = launch_gemm(s, true, st, err, s->d_coef2, 1);
    if (rc) return rc;
    T->end(st);
    // F0 + the correction, added as the permutation reads them
    T->begin(ST_BASIS, st);
    group_to_packed_tiled<<<ptile_grid(s->L, s->batch), 256, 0, st>>>(s->d_fg, (float2*)coeffs, s->d_goff2, s->L,
                                                                      coeffs_per_fn(s), s->batch, s->d_coef2);
    TCK(cudaGetLastError());
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_refine_add_pencils(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    if (!s->refine || !s->d_coef2 || s->s2) {
        err = "internal: refinement buffers were not allocated";
        return FFTSO3_ERR_CUDA;
    }
    // the correction in the coefficients' own element type: complex in d_coef2, real kinds in d_fc; its GEMM with
    // one BF16 term (the residual is small: see tc_refine_finish_group)
    void* corr = s->real ? (void*)s->d_fc : (void*)s->d_coef2;
    if (s->real) {
        // tc_forward_finish writes the complex coefficients into d_fc first; route them through d_coef2
        T->begin(ST_GEMM_FWD, st);
        int rc = launch_gemm(s, true, st, err, nullptr, 1);
        if (rc) return rc;
        T->end(st);
        T->begin(ST_BASIS, st);
        group_to_packed_tiled<<<ptile_grid(s->L, s->batch), 256, 0, st>>>(s->d_fg, s->d_coef2, s->d_goff2, s->L,
                                                                          coeffs_per_fn(s), s->batch);
        TCK(cudaGetLastError());
        TCK(launch_so3_c2r(s->d_coef2, s->d_fc, false, s->L, s->batch, st));
        T->end(st);
    } else {
        int rc = forward_from_pencils(s, s->d_coef2, st, T, err, 1);
        if (rc) return rc;
    }
    const long long nc = (long long)s->batch * coeffs_per_fn(s);
    T->begin(ST_REFINE, st);
    TCK(launch_add_real((float*)coeffs, (const float*)corr, s->real ? nc : 2 * nc, st));
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_refine_add(TCState* s, const void* resid, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    if (!s->refine || !s->d_coef2) {
        err = "internal: refinement buffers were not allocated";
        return FFTSO3_ERR_CUDA;
    }
    const long long nc = (long long)s->batch * coeffs_per_fn(s);
    int rc;
    float* corr;  // the correction in the coefficients' own element type
    if (s->real && s->s2) {
        rc = tc_forward_once(s, resid, nullptr, st, T, err, s->d_coef2);
        corr = (float*)s->d_coef2;
    } else {
        rc = tc_forward_once(s, resid, s->d_coef2, st, T, err);
        corr = (float*)s->d_coef2;
        if (!rc && s->real) {
            // real basis of the correction, into the (complex-sized) scratch d_fc
            T->begin(ST_BASIS, st);
            if (s->s2)
                TCK(launch_s2_c2r(s->d_coef2, s->d_fc, false, s->L, s->batch, st));
            else
                TCK(launch_so3_c2r(s->d_coef2, s->d_fc, false, s->L, s->batch, st));
            T->end(st);
            corr = (float*)s->d_fc;
        }
    }
    if (rc) return rc;
    T->begin(ST_REFINE, st);
    TCK(launch_add_real((float*)coeffs, corr, s->real ? nc : 2 * nc, st));
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_inverse(TCState* s, const void* coeffs, void* grid, cudaStream_t st, StageTimer* T, std::string& err)
{
    if (s->real && s->s2) return tc_inverse_once(s, nullptr, grid, st, T, err, coeffs);
    const float2* Fc = (const float2*)coeffs;
    if (s->real) {
        T->begin(ST_BASIS, st);
        if (s->s2)
            TCK(launch_s2_r2c(coeffs, s->d_fc, false, s->L, s->batch, st));
        else
            TCK(launch_so3_r2c(coeffs, s->d_fc, false, s->L, s->batch, st));
        T->end(st);
        Fc = s->d_fc;
    }
    return tc_inverse_once(s, Fc, grid, st, T, err);
}

// ---- phases of one direction, for launches fused across plans

int tc_forward_fft(TCState* s, const void* grid, cudaStream_t st, StageTimer* T, std::string& err)
{
    return fft_forward(s, grid, st, T, err);
}

int tc_forward_finish(TCState* s, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    float2* Fc = s->real ? s->d_fc : (float2*)coeffs;
    T->begin(ST_BASIS, st);
    if (s->real && s->s2) {
        TCK(launch_s2_group_to_real(s->d_fg, coeffs, s->d_goff2, s->L, s->batch, st));
        T->end(st);
        return FFTSO3_SUCCESS;
    }
    if (s->s2)
        s2_group_to_packed_kernel<<<dim3(s->B, s->batch), 256, 0, st>>>(s->d_fg, Fc, s->d_goff2, s->L,
                                                                       coeffs_per_fn(s));
    else
        group_to_packed_tiled<<<ptile_grid(s->L, s->batch), 256, 0, st>>>(s->d_fg, Fc, s->d_goff2, s->L,
                                                                    coeffs_per_fn(s), s->batch);
    TCK(cudaGetLastError());
    if (s->real) {
        if (s->s2)
            TCK(launch_s2_c2r(Fc, coeffs, false, s->L, s->batch, st));
        else
            TCK(launch_so3_c2r(Fc, coeffs, false, s->L, s->batch, st));
    }
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_inverse_prepare(TCState* s, const void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    const float2* Fc = (const float2*)coeffs;
    const long long N = s->N;
    T->begin(ST_BASIS, st);
    if (s->real && s->s2) {
        const long long tot = (long long)s->batch * N;
        s2_zero_nyquist_pencils_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(s->d_pencil, (int)N, s->batch);
        TCK(cudaGetLastError());
        TCK(launch_s2_real_to_group(coeffs, s->d_fg, s->d_goff2, s->L, s->batch, st));
        T->end(st);
        return FFTSO3_SUCCESS;
    }
    if (s->real) {
        if (s->s2)
            TCK(launch_s2_r2c(coeffs, s->d_fc, false, s->L, s->batch, st));
        else
            TCK(launch_so3_r2c(coeffs, s->d_fc, false, s->L, s->batch, st));
        Fc = s->d_fc;
    }
    if (s->s2) {
        const long long tot = (long long)s->batch * N;
        s2_zero_nyquist_pencils_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(s->d_pencil, (int)N, s->batch);
        s2_packed_to_group_kernel<<<dim3(s->ngroups, s->batch), 128, 0, st>>>(Fc, s->d_fg, s->d_goff2, s->L,
                                                                             coeffs_per_fn(s));
    } else {
        const long long tot = (long long)s->batch * 2 * N * N;
        zero_nyquist_pencils_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(s->d_pencil, (int)N, s->batch);
        packed_to_group_tiled<<<ptile_grid(s->L, s->batch), 256, 0, st>>>(Fc, s->d_fg, s->d_goff2, s->L,
                                                                          coeffs_per_fn(s), s->batch);
    }
    TCK(cudaGetLastError());
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_inverse_fft(TCState* s, void* grid, cudaStream_t st, StageTimer* T, std::string& err)
{
    return fft_inverse(s, grid, st, T, err);
}

struct TCFused {
    std::vector<TCState*> parts;
    GemmSeg* d_segs[2] = {nullptr, nullptr};  // forward, inverse
    int4* d_items[2] = {nullptr, nullptr};
    int2* d_iaux[2] = {nullptr, nullptr};
    int nitems[2] = {0, 0};
    int* d_err = nullptr;
    int nsm = 0;
    bool s2 = false;
    // three-launch directions (SO(3) batches, tc_fused_phases): the bucket table of the slice FFT and the
    // coefficient conversions
    BucketSeg* d_bseg = nullptr;
    unsigned short* d_cseg = nullptr;  // segment of each conversion CTA
    int nbseg = 0;
    long long nblk = 0, ncblk = 0;
    size_t slice_smem = 0;
    bool real = false;
    bool slice_wide = false;  // 512-thread slice FFT CTAs (FFTSO3_SLICE_WIDE=1)
};

void tc_fused_destroy(TCFused* f)
{
    if (!f) return;
    if (f->d_bseg) cudaFree(f->d_bseg);
    if (f->d_cseg) cudaFree(f->d_cseg);
    for (int d = 0; d < 2; ++d) {
        if (f->d_segs[d]) cudaFree(f->d_segs[d]);
        if (f->d_items[d]) cudaFree(f->d_items[d]);
        if (f->d_iaux[d]) cudaFree(f->d_iaux[d]);
    }
    if (f->d_err) cudaFree(f->d_err);
    delete f;
}

// One work list over the tensor-core plans `parts` (same kind, at most 32768
// plans): items of plan i carry segment i; sorted by decreasing k-steps so the
// longest items start first on the persistent CTAs.
int tc_fused_create(TCFused** out, const std::vector<TCState*>& parts, std::string& err)
{
    *out = nullptr;
    if (parts.empty() || parts.size() > 32768) {
        err = "fused launch: 1 to 32768 plans";
        return FFTSO3_ERR_INVALID_ARG;
    }
    for (TCState* p : parts)
        if (!p || p->simt || p->s2 != parts[0]->s2 || p->ntiles > 0xFFFF) {
            err = "fused launch: all plans must be tensor-core plans of one family (SO(3) or S^2)";
            return FFTSO3_ERR_INVALID_ARG;
        }
    TCFused* f = new TCFused();
    f->parts = parts;
    f->s2 = parts[0]->s2;
    f->nsm = parts[0]->nsm;
    auto fail = [&](cudaError_t e, const char* what) {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        tc_fused_destroy(f);
        return FFTSO3_ERR_CUDA;
    };
    cudaError_t e;
    for (int d = 0; d < 2; ++d) {
        const bool fwd = d == 0;
        std::vector<GemmSeg> segs(parts.size());
        struct FItem {
            int nk;
            int4 it;
            int2 aux;
        };
        std::vector<FItem> items;
        for (size_t i = 0; i < parts.size(); ++i) {
            TCState* p = parts[i];
            GemmArgs a = gemm_args(p);
            if (fwd) {
                a.pin = p->d_pencil;
                a.cout = p->d_fg;
            } else {
                a.cin = p->d_fg;
                a.pout = p->d_pencil;
            }
            segs[i].a = a;
            for (int q = 0; q < 3; ++q) segs[i].tm[q] = fwd ? p->tmA_fwd[q] : p->tmA_inv[q];
            for (size_t j = 0; j < p->items_h[d].size(); ++j) {
                const int4& it = p->items_h[d][j];
                const int m0 = it.w >> 16;
                const int nk = fwd ? p->Kp / BK : (p->B - m0 + BK - 1) / BK;
                items.push_back({nk, make_int4(it.x, it.y, ((int)i << 16) | it.z, it.w), p->iaux_h[d][j]});
            }
        }
        std::stable_sort(items.begin(), items.end(), [](const FItem& a, const FItem& b) { return a.nk > b.nk; });
        std::vector<int4> flat(items.size());
        std::vector<int2> faux(items.size());
        for (size_t i = 0; i < items.size(); ++i) {
            flat[i] = items[i].it;
            faux[i] = items[i].aux;
        }
        f->nitems[d] = (int)flat.size();
        if ((e = cudaMalloc(&f->d_segs[d], sizeof(GemmSeg) * segs.size())) != cudaSuccess) return fail(e, "cudaMalloc");
        if ((e = cudaMalloc(&f->d_items[d], sizeof(int4) * std::max<size_t>(flat.size(), 1))) != cudaSuccess)
            return fail(e, "cudaMalloc");
        if ((e = cudaMemcpy(f->d_segs[d], segs.data(), sizeof(GemmSeg) * segs.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
            return fail(e, "cudaMemcpy");
        if (!flat.empty() && (e = cudaMemcpy(f->d_items[d], flat.data(), sizeof(int4) * flat.size(),
                                             cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "cudaMemcpy");
        if ((e = cudaMalloc(&f->d_iaux[d], sizeof(int2) * std::max<size_t>(faux.size(), 1))) != cudaSuccess)
            return fail(e, "cudaMalloc");
        if (!faux.empty() && (e = cudaMemcpy(f->d_iaux[d], faux.data(), sizeof(int2) * faux.size(),
                                             cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "cudaMemcpy");
    }
    if ((e = cudaMalloc(&f->d_err, sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc");
    cudaMemset(f->d_err, 0, sizeof(int));
    *out = f;
    return FFTSO3_SUCCESS;
}

// The beta-sum GEMM of every plan of `f` in one persistent launch.
int tc_fused_gemm(TCFused* f, bool fwd, cudaStream_t st, StageTimer* T, std::string& err)
{
    const int d = fwd ? 0 : 1;
    if (f->nitems[d] == 0) return FFTSO3_SUCCESS;
    GemmArgs a = gemm_args(f->parts[0]);
    a.items = f->d_items[d];
    a.iaux = f->d_iaux[d];
    a.nitems = f->nitems[d];
    a.err = f->d_err;
    const int nctas = a.nitems < f->nsm ? a.nitems : f->nsm;
    const CUtensorMap* tm = fwd ? f->parts[0]->tmA_fwd : f->parts[0]->tmA_inv;  // unused by fused kernels
    T->begin(fwd ? ST_GEMM_FWD : ST_GEMM_INV, st);
    if (fwd && f->s2)
        so3_tc_gemm_kernel<true, true, true><<<nctas, THREADS, SMEM_BYTES, st>>>(tm[0], tm[1], tm[2], a, f->d_segs[d]);
    else if (fwd)
        so3_tc_gemm_kernel<true, false, true><<<nctas, THREADS, SMEM_BYTES, st>>>(tm[0], tm[1], tm[2], a, f->d_segs[d]);
    else if (f->s2)
        so3_tc_gemm_kernel<false, true, true><<<nctas, THREADS, SMEM_BYTES, st>>>(tm[0], tm[1], tm[2], a, f->d_segs[d]);
    else
        so3_tc_gemm_kernel<false, false, true><<<nctas, THREADS, SMEM_BYTES, st>>>(tm[0], tm[1], tm[2], a, f->d_segs[d]);
    TCK(cudaGetLastError());
    T->end(st);
    return FFTSO3_SUCCESS;
}

// The bucket table of the three-launch directions.  Buckets run longest slices first (descending N) in both
// the slice FFT and the conversions; a CTA of the slice FFT takes as many slices of its bucket as the launch's
// shared memory (sized for one slice of the largest N) holds, up to about the largest slice's sample count, so
// small bandwidths get as much work per CTA as large ones.
int tc_fused_phases(TCFused* f, const std::vector<long long>& g0, const std::vector<long long>& c0, std::string& err)
{
    const size_t n = f->parts.size();
    if (f->s2 || g0.size() != n || c0.size() != n) {
        err = "fused phases: SO(3) plans with one grid and one coefficient offset each";
        return FFTSO3_ERR_UNSUPPORTED;
    }
    const bool real = f->parts[0]->real;
    const char* ev_wide = getenv("FFTSO3_SLICE_WIDE");
    const bool wide = ev_wide && ev_wide[0] == '1';
    int Nmax = 0;
    size_t smem = 0;
    for (TCState* p : f->parts) {
        if (p->real != real || p->refine || p->simt) {
            err = "fused phases: tensor-core plans of one kind without refinement";
            return FFTSO3_ERR_UNSUPPORTED;
        }
        Nmax = std::max(Nmax, p->N);
        smem = std::max(smem, slice_fft_smem_bytes(p->N, 1, real, wide));
    }
    int maxsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem > (size_t)maxsm) {
        err = "fused phases: one beta slice of N = " + std::to_string(Nmax) + " exceeds the shared memory of a CTA";
        return FFTSO3_ERR_UNSUPPORTED;
    }
    std::vector<int> ord(n);
    for (size_t i = 0; i < n; ++i) ord[i] = (int)i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return f->parts[a]->N > f->parts[b]->N; });
    std::vector<BucketSeg> segs;
    long long blk = 0, cblk = 0;
    for (int i : ord) {
        TCState* p = f->parts[i];
        const int N = p->N;
        BucketSeg s{};
        s.L = p->L;
        s.B = p->B;
        s.N = N;
        s.batch = p->batch;
        s.G = slice_lines_per_group(N, wide);
        int spc = 1;
        while (spc < 256 && slice_fft_smem_bytes(N, spc + 1, real, wide) <= smem &&
               (long long)(spc + 1) * N * N <= (long long)Nmax * Nmax)
            ++spc;
        s.spc = spc;
        s.fac = p->fac;
        s.tw = reinterpret_cast<const double2*>(p->d_tw);
        s.pencil = p->d_pencil;
        s.fg = p->d_fg;
        s.g0 = g0[i];
        s.c0 = c0[i];
        s.blk0 = blk;
        s.cblk0 = cblk;
        blk += ((long long)p->batch * N + spc - 1) / spc;
        cblk += ((long long)p->batch * so3_off(p->B) + CONVERT_THREADS - 1) / CONVERT_THREADS;
        segs.push_back(s);
    }
    if (segs.size() > 65535 || Nmax > 512) {
        err = "fused phases: at most 65535 buckets of l_max <= 255";
        return FFTSO3_ERR_UNSUPPORTED;
    }
    std::vector<unsigned short> cseg((size_t)cblk);
    for (size_t i = 0; i < segs.size(); ++i) {
        const long long end = i + 1 < segs.size() ? segs[i + 1].cblk0 : cblk;
        for (long long c = segs[i].cblk0; c < end; ++c) cseg[(size_t)c] = (unsigned short)i;
    }
    cudaError_t e;
    if (f->d_bseg) cudaFree(f->d_bseg);
    if (f->d_cseg) cudaFree(f->d_cseg);
    f->d_bseg = nullptr;
    f->d_cseg = nullptr;
    if ((e = cudaMalloc(&f->d_bseg, sizeof(BucketSeg) * segs.size())) != cudaSuccess ||
        (e = cudaMemcpy(f->d_bseg, segs.data(), sizeof(BucketSeg) * segs.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (e = cudaMalloc(&f->d_cseg, sizeof(unsigned short) * std::max<size_t>(cseg.size(), 1))) != cudaSuccess ||
        (!cseg.empty() && (e = cudaMemcpy(f->d_cseg, cseg.data(), sizeof(unsigned short) * cseg.size(),
                                          cudaMemcpyHostToDevice)) != cudaSuccess)) {
        err = std::string("fused phases: ") + cudaGetErrorString(e);
        return FFTSO3_ERR_CUDA;
    }
    f->nbseg = (int)segs.size();
    f->nblk = blk;
    f->ncblk = cblk;
    f->slice_smem = smem;
    f->real = real;
    f->slice_wide = wide;
    return FFTSO3_SUCCESS;
}

int tc_fused_forward(TCFused* f, const void* grid, void* coeffs, cudaStream_t st, StageTimer* T, std::string& err)
{
    if (!f->d_bseg) {
        err = "internal: fused phases were not set up";
        return FFTSO3_ERR_CUDA;
    }
    T->begin(ST_FFT_SLICES, st);
    TCK(launch_slice_fft(f->d_bseg, f->nbseg, f->nblk, f->slice_smem, true, f->real, f->slice_wide, grid, nullptr, st));
    T->end(st);
    int rc = tc_fused_gemm(f, true, st, T, err);
    if (rc) return rc;
    T->begin(ST_CONVERT, st);
    TCK(launch_fused_group_to_packed(f->d_bseg, f->d_cseg, f->ncblk, f->real, coeffs, st));
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_fused_inverse(TCFused* f, const void* coeffs, void* grid, cudaStream_t st, StageTimer* T, std::string& err)
{
    if (!f->d_bseg) {
        err = "internal: fused phases were not set up";
        return FFTSO3_ERR_CUDA;
    }
    T->begin(ST_CONVERT, st);
    TCK(launch_fused_packed_to_group(f->d_bseg, f->d_cseg, f->ncblk, f->real, coeffs, st));
    T->end(st);
    int rc = tc_fused_gemm(f, false, st, T, err);
    if (rc) return rc;
    T->begin(ST_FFT_SLICES, st);
    TCK(launch_slice_fft(f->d_bseg, f->nbseg, f->nblk, f->slice_smem, false, f->real, f->slice_wide, nullptr, grid, st));
    T->end(st);
    return FFTSO3_SUCCESS;
}

int tc_fused_status(TCFused* f)
{
    int h = 0;
    if (cudaMemcpy(&h, f->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h;
}

int tc_status(TCState* s)
{
    int h = 0;
    if (cudaMemcpy(&h, s->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h;
}

}  // namespace fftso3
