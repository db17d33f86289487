// Batches of functions of uneven bandwidth (fftso3_batch_*, include/fftso3_gb300.h).
//
// The reference transforms one function per call (FFTSO3_real::forward_transform,
// fdcl_FFTSO3.cpp:774-850; inverse_transform, :1141-1167); a user with many
// functions of different l_max loops over them, re-initialising the object
// whenever l_max changes (:500).  Here the whole set is one object:
//
//  * functions are bucketed by l_max; each bucket is an ordinary plan with
//    batch = the bucket's size, so every stage runs batched over its
//    functions (the tensor-core beta-sum is a GEMM over the function batch);
//  * the plan decides where each function lives in the caller's buffers:
//    bucket-major (ascending l_max), caller order inside a bucket, so that a
//    bucket is one contiguous slab and no gather/scatter pass is needed.
//    fftso3_batch_grid_offset / fftso3_batch_coeff_offset give the place;
//  * buckets are spread over a few internal streams (longest work first, each
//    bucket to the least-loaded stream) forked from and joined back into the
//    caller's stream, so small bandwidths run side by side on the SMs;
//  * tensor-core batches without refinement run the beta-sum GEMM of all
//    buckets as ONE persistent launch (tc_fused_gemm: one work list over every
//    bucket's (group, row tile, column tile) items, longest first): forward =
//    fork / per-bucket FFTs / join / fused GEMM / fork / per-bucket coefficient
//    permutations / join, inverse the mirror image;
//  * SO(3) tensor-core batches without refinement go further: each direction is
//    three launches over all buckets (fused.cuh) -- one slice-FFT launch (every
//    bucket's beta slices, a CTA per slice or per few slices), the fused GEMM,
//    one coefficient-conversion launch -- on the caller's stream, no fork/join;
//  * with FFTSO3_FLAG_GRAPH the whole fork / bucket launches / join sequence
//    is captured once per (direction, input, output) into a CUDA graph and
//    replayed with one cudaGraphLaunch afterwards, which removes the
//    per-launch host cost of the several hundred small launches.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/fftso3_gb300.h"
#include "common.cuh"
#include "fused.cuh"
#include "tc.cuh"

using namespace fftso3;

namespace {

constexpr int MAX_STREAMS = 8;

int bfail(int code, const std::string& m)
{
    set_last_error(m);
    return code;
}

int bcuda(cudaError_t e, const char* what)
{
    return bfail(FFTSO3_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool kind_is_so3(int k) { return k == FFTSO3_SO3_COMPLEX || k == FFTSO3_SO3_REAL; }
bool kind_is_real(int k) { return k == FFTSO3_SO3_REAL || k == FFTSO3_S2_REAL; }

}  // namespace

struct fftso3_batch {
    int device = 0, kind = 0, precision = 0, recursion = 0, n = 0;
    unsigned flags = 0;
    size_t gbytes = 0, cbytes = 0;               // bytes per grid / coefficient element
    std::vector<long long> goff, coff;           // per function, in elements (n + 1 entries)
    struct Bucket {
        int L = 0, count = 0, stream = 0;
        long long g0 = 0, c0 = 0;                // element offsets of the bucket's slab
        double cost = 0;
        fftso3_plan* plan = nullptr;
    };
    std::vector<Bucket> buckets;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> joined;
    cudaEvent_t fork = nullptr;
    cudaStream_t capture = nullptr;
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        const void* in = nullptr;
        void* out = nullptr;
        int kernels = -1;                        // kernel nodes of the captured graph
    } graphs[2];
    long long bytes = 0;
    bool timing = false;                         // per-stage timing (eager launches, no graph)
    bool tuned = false;                          // stream count chosen (FFTSO3_FLAG_AUTOTUNE)
    int nstreams_used = 0;
    TCFused* fused = nullptr;                    // one GEMM launch over all buckets
    bool phases = false;                         // SO(3): three launches per direction over all buckets
    StageTimer timer;                            // the fused launches' stage times
};

namespace {

void batch_free(fftso3_batch* b)
{
    if (b->fused) tc_fused_destroy(b->fused);
    b->timer.enabled = false;
    b->timer.collect();
    for (auto& g : b->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (auto& k : b->buckets)
        if (k.plan) fftso3_plan_destroy(k.plan);
    for (cudaEvent_t e : b->joined)
        if (e) cudaEventDestroy(e);
    for (cudaStream_t s : b->streams)
        if (s) cudaStreamDestroy(s);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->capture) cudaStreamDestroy(b->capture);
}

int check_batch(const fftso3_batch* b)
{
    if (!b) return bfail(FFTSO3_ERR_INVALID_ARG, "batch is NULL");
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != b->device) {
        cudaError_t e = cudaSetDevice(b->device);
        if (e != cudaSuccess) return bcuda(e, "cudaSetDevice");
    }
    return FFTSO3_SUCCESS;
}

// buckets to ns streams: longest work first, each to the least-loaded stream
void assign_streams(fftso3_batch* b, int ns)
{
    std::vector<double> load(ns, 0.0);
    std::vector<int> byc(b->buckets.size());
    std::iota(byc.begin(), byc.end(), 0);
    std::stable_sort(byc.begin(), byc.end(),
                     [&](int a, int c) { return b->buckets[a].cost > b->buckets[c].cost; });
    for (int i : byc) {
        const int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        b->buckets[i].stream = s;
        load[s] += b->buckets[i].cost;
    }
    b->nstreams_used = ns;
}

int launch_all(fftso3_batch* b, int dir, const void* in, void* out, cudaStream_t st);

// FFTSO3_FLAG_AUTOTUNE: time 1, 2, 4, 8 bucket streams on this call's own
// buffers (one warm-up and one timed eager run each; the real call follows and
// overwrites the output) and keep the fastest.
int tune_streams(fftso3_batch* b, int dir, const void* in, void* out, cudaStream_t st)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bestn = (int)b->streams.size();
    for (int ns = 1; ns <= (int)b->streams.size(); ns *= 2) {
        assign_streams(b, ns);
        int rc = launch_all(b, dir, in, out, st);
        if (!rc) {
            cudaEventRecord(e0, st);
            rc = launch_all(b, dir, in, out, st);
            cudaEventRecord(e1, st);
        }
        if (rc || cudaEventSynchronize(e1) != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return rc ? rc : bcuda(cudaGetLastError(), "autotune");
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            bestn = ns;
        }
    }
    assign_streams(b, bestn);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->tuned = true;
    return FFTSO3_SUCCESS;
}

int fork_from(fftso3_batch* b, cudaStream_t st)
{
    cudaError_t e;
    if ((e = cudaEventRecord(b->fork, st)) != cudaSuccess) return bcuda(e, "cudaEventRecord");
    for (cudaStream_t s : b->streams)
        if ((e = cudaStreamWaitEvent(s, b->fork, 0)) != cudaSuccess) return bcuda(e, "cudaStreamWaitEvent");
    return FFTSO3_SUCCESS;
}

int join_into(fftso3_batch* b, cudaStream_t st)
{
    cudaError_t e;
    for (size_t i = 0; i < b->streams.size(); ++i) {
        if ((e = cudaEventRecord(b->joined[i], b->streams[i])) != cudaSuccess) return bcuda(e, "cudaEventRecord");
        if ((e = cudaStreamWaitEvent(st, b->joined[i], 0)) != cudaSuccess) return bcuda(e, "cudaStreamWaitEvent");
    }
    return FFTSO3_SUCCESS;
}

// phase 0 (before the fused GEMM) or 1 (after it) of one bucket
int bucket_phase(fftso3_batch* b, const fftso3_batch::Bucket& k, int dir, int phase, const void* pin, void* pout,
                 cudaStream_t s)
{
    TCState* tc = plan_tc_state(k.plan);
    StageTimer* T = plan_timer(k.plan);
    std::string err;
    int rc;
    if (dir == 0)
        rc = phase == 0 ? tc_forward_fft(tc, pin, s, T, err) : tc_forward_finish(tc, pout, s, T, err);
    else
        rc = phase == 0 ? tc_inverse_prepare(tc, pin, s, T, err) : tc_inverse_fft(tc, pout, s, T, err);
    if (rc) return bfail(rc, err);
    return FFTSO3_SUCCESS;
}

// fork from `st`, every bucket on its stream, join back into `st` (with a
// fused GEMM: twice, around the one GEMM launch on `st`)
int launch_all(fftso3_batch* b, int dir, const void* in, void* out, cudaStream_t st)
{
    int rc;
    const size_t isz = dir == 0 ? b->gbytes : b->cbytes, osz = dir == 0 ? b->cbytes : b->gbytes;
    auto ptrs = [&](const fftso3_batch::Bucket& k, const void*& pin, void*& pout) {
        const long long i0 = dir == 0 ? k.g0 : k.c0, o0 = dir == 0 ? k.c0 : k.g0;
        pin = (const char*)in + (size_t)i0 * isz;
        pout = (char*)out + (size_t)o0 * osz;
    };
    // timing mode runs the buckets one after another on the caller's stream (exact stage times)
    auto sof = [&](const fftso3_batch::Bucket& k) { return b->timing ? st : b->streams[k.stream]; };
    if (b->phases) {
        std::string err;
        rc = dir == 0 ? tc_fused_forward(b->fused, in, out, st, &b->timer, err)
                      : tc_fused_inverse(b->fused, in, out, st, &b->timer, err);
        return rc ? bfail(rc, err) : FFTSO3_SUCCESS;
    }
    if ((rc = fork_from(b, st))) return rc;
    if (!b->fused) {
        for (const auto& k : b->buckets) {
            const void* pin;
            void* pout;
            ptrs(k, pin, pout);
            rc = dir == 0 ? fftso3_forward(k.plan, pin, pout, sof(k)) : fftso3_inverse(k.plan, pin, pout, sof(k));
            if (rc) return rc;
        }
        return join_into(b, st);
    }
    for (const auto& k : b->buckets) {
        const void* pin;
        void* pout;
        ptrs(k, pin, pout);
        if ((rc = bucket_phase(b, k, dir, 0, pin, pout, sof(k)))) return rc;
    }
    if ((rc = join_into(b, st))) return rc;
    {
        std::string err;
        if ((rc = tc_fused_gemm(b->fused, dir == 0, st, &b->timer, err))) return bfail(rc, err);
    }
    if ((rc = fork_from(b, st))) return rc;
    for (const auto& k : b->buckets) {
        const void* pin;
        void* pout;
        ptrs(k, pin, pout);
        if ((rc = bucket_phase(b, k, dir, 1, pin, pout, sof(k)))) return rc;
    }
    return join_into(b, st);
}

int run(fftso3_batch* b, int dir, const void* in, void* out, void* stream)
{
    int rc = check_batch(b);
    if (rc) return rc;
    if (!in || !out) return bfail(FFTSO3_ERR_INVALID_ARG, "input/output pointer is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    if ((b->flags & FFTSO3_FLAG_AUTOTUNE) && !b->tuned && !b->timing && !b->phases)
        if ((rc = tune_streams(b, dir, in, out, st))) return rc;
    if (!(b->flags & FFTSO3_FLAG_GRAPH) || b->timing) return launch_all(b, dir, in, out, st);

    auto& g = b->graphs[dir];
    if (!g.exec || g.in != in || g.out != out) {
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        // captured on an internal stream, so the caller's stream may be the legacy default stream
        cudaError_t e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) return bcuda(e, "cudaStreamBeginCapture");
        rc = launch_all(b, dir, in, out, b->capture);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(b->capture, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return bcuda(e, "cudaStreamEndCapture");
        {
            size_t nn = 0;
            g.kernels = -1;
            if (cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess) {
                std::vector<cudaGraphNode_t> nodes(nn);
                if (nn == 0 || cudaGraphGetNodes(graph, nodes.data(), &nn) == cudaSuccess) {
                    int nk = 0;
                    for (size_t i = 0; i < nn; ++i) {
                        cudaGraphNodeType t;
                        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++nk;
                    }
                    g.kernels = nk;
                }
            }
        }
        e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            g.exec = nullptr;
            return bcuda(e, "cudaGraphInstantiate");
        }
        g.in = in;
        g.out = out;
    }
    cudaError_t e = cudaGraphLaunch(g.exec, st);
    if (e != cudaSuccess) return bcuda(e, "cudaGraphLaunch");
    return FFTSO3_SUCCESS;
}

}  // namespace

extern "C" {

int fftso3_batch_create(fftso3_batch** out, int kind, const int* l_max, int n_functions, int precision,
                        int recursion, unsigned flags)
{
    if (!out) return bfail(FFTSO3_ERR_INVALID_ARG, "batch output pointer is NULL");
    *out = nullptr;
    if (!l_max) return bfail(FFTSO3_ERR_INVALID_ARG, "l_max array is NULL");
    if (n_functions < 1) return bfail(FFTSO3_ERR_INVALID_ARG, "n_functions must be >= 1");
    if ((flags & ~(FFTSO3_FLAG_REFINE | FFTSO3_FLAG_GRAPH | FFTSO3_FLAG_AUTOTUNE)) != 0)
        return bfail(FFTSO3_ERR_INVALID_ARG, "unknown flag bits");
    if (kind < FFTSO3_SO3_COMPLEX || kind > FFTSO3_S2_REAL)
        return bfail(FFTSO3_ERR_INVALID_ARG, "unknown transform kind");
    if (precision != FFTSO3_PREC_FP64 && precision != FFTSO3_PREC_TC_BF16X3 && precision != FFTSO3_PREC_FP32)
        return bfail(FFTSO3_ERR_INVALID_ARG, "unknown precision");
    for (int i = 0; i < n_functions; ++i)
        if (l_max[i] < 0)
            return bfail(FFTSO3_ERR_INVALID_ARG, "l_max[" + std::to_string(i) + "] must be >= 0");

    fftso3_batch* b = new fftso3_batch();
    b->kind = kind;
    b->precision = precision;
    b->recursion = recursion;
    b->n = n_functions;
    b->flags = flags;
    cudaGetDevice(&b->device);
    const bool fp64 = precision == FFTSO3_PREC_FP64, real = kind_is_real(kind);
    b->gbytes = real ? (fp64 ? 8 : 4) : (fp64 ? 16 : 8);
    b->cbytes = b->gbytes;
    auto bail = [&](int rc) {
        batch_free(b);
        delete b;
        return rc;
    };

    // buckets in ascending l_max; offsets bucket-major, caller order inside a bucket
    std::vector<int> order(n_functions);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return l_max[a] < l_max[c]; });
    b->goff.assign(n_functions + 1, 0);
    b->coff.assign(n_functions + 1, 0);
    long long g = 0, c = 0;
    for (int i = 0; i < n_functions; ++i) {
        const int f = order[i], L = l_max[f];
        if (b->buckets.empty() || b->buckets.back().L != L) {
            fftso3_batch::Bucket k;
            k.L = L;
            k.g0 = g;
            k.c0 = c;
            b->buckets.push_back(k);
        }
        b->buckets.back().count++;
        b->goff[f] = g;
        b->coff[f] = c;
        g += fftso3_grid_elems(kind, L);
        c += fftso3_coeff_elems(kind, L);
    }
    b->goff[n_functions] = g;
    b->coff[n_functions] = c;

    // SO(3) tensor-core batches without refinement run each direction as three launches over all buckets
    // (slice FFT, GEMM, conversion) when one beta slice of the largest bandwidth fits a CTA's shared memory;
    // their bucket plans then need no tuned FFT launch shapes.  FFTSO3_BATCH_PHASES=0 keeps the per-bucket
    // phases around the fused GEMM.
    bool want_phases = false;
    if (precision == FFTSO3_PREC_TC_BF16X3 && !(flags & FFTSO3_FLAG_REFINE) && kind_is_so3(kind)) {
        const char* ev = std::getenv("FFTSO3_BATCH_PHASES");
        int maxsm = 0;
        cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
        want_phases = !(ev && ev[0] == '0') &&
                      slice_fft_smem_bytes(2 * (b->buckets.back().L + 1), 1, real, false) <= (size_t)maxsm;
    }
    unsigned pflags = flags & (FFTSO3_FLAG_REFINE | FFTSO3_FLAG_AUTOTUNE);
    if (want_phases) pflags &= ~FFTSO3_FLAG_AUTOTUNE;

    // one plan per bucket
    for (auto& k : b->buckets) {
        int rc = fftso3_plan_create(&k.plan, kind, k.L, k.count, precision, recursion, pflags);
        if (rc) {
            k.plan = nullptr;
            std::string m = fftso3_last_error_string();
            bail(rc);
            return bfail(rc, "bucket l_max=" + std::to_string(k.L) + ": " + m);
        }
        b->bytes += fftso3_plan_device_bytes(k.plan);
        const double N = 2.0 * (k.L + 1);
        k.cost = (double)k.count * (kind_is_so3(kind) ? N * N * N : N * N) * std::log2(N);
    }

    // streams: longest bucket first, each to the least-loaded stream
    const int ns = std::min<int>(MAX_STREAMS, (int)b->buckets.size());
    assign_streams(b, ns);
    cudaError_t e;
    b->streams.assign(ns, nullptr);
    b->joined.assign(ns, nullptr);
    for (int s = 0; s < ns; ++s) {
        if ((e = cudaStreamCreateWithFlags(&b->streams[s], cudaStreamNonBlocking)) != cudaSuccess)
            return bail(bcuda(e, "cudaStreamCreateWithFlags"));
        if ((e = cudaEventCreateWithFlags(&b->joined[s], cudaEventDisableTiming)) != cudaSuccess)
            return bail(bcuda(e, "cudaEventCreateWithFlags"));
    }
    if ((e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess)
        return bail(bcuda(e, "cudaEventCreateWithFlags"));
    if ((e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(bcuda(e, "cudaStreamCreateWithFlags"));
    if (precision == FFTSO3_PREC_TC_BF16X3 && !(flags & FFTSO3_FLAG_REFINE)) {
        std::vector<TCState*> parts;
        for (auto& k : b->buckets) parts.push_back(plan_tc_state(k.plan));
        std::string err;
        int rc = tc_fused_create(&b->fused, parts, err);
        if (!rc && want_phases) {
            std::vector<long long> g0, c0;
            for (auto& k : b->buckets) {
                g0.push_back(k.g0);
                c0.push_back(k.c0);
            }
            rc = tc_fused_phases(b->fused, g0, c0, err);
            if (rc == FFTSO3_SUCCESS) {
                b->phases = true;
                b->tuned = true;
                b->nstreams_used = 1;
            } else if (rc == FFTSO3_ERR_UNSUPPORTED) {
                rc = FFTSO3_SUCCESS;
            }
        }
        if (rc) {
            bail(rc);
            return bfail(rc, err);
        }
    }
    *out = b;
    return FFTSO3_SUCCESS;
}

int fftso3_batch_destroy(fftso3_batch* b)
{
    if (!b) return bfail(FFTSO3_ERR_INVALID_ARG, "batch is NULL");
    int dev = -1;
    cudaGetDevice(&dev);
    const int bdev = b->device;
    if (dev != bdev) cudaSetDevice(bdev);
    batch_free(b);
    delete b;
    if (dev >= 0 && dev != bdev) cudaSetDevice(dev);
    return FFTSO3_SUCCESS;
}

long long fftso3_batch_grid_offset(const fftso3_batch* b, int fn)
{
    if (!b || fn < 0 || fn > b->n) return -1;
    return b->goff[fn];
}

long long fftso3_batch_coeff_offset(const fftso3_batch* b, int fn)
{
    if (!b || fn < 0 || fn > b->n) return -1;
    return b->coff[fn];
}

int fftso3_batch_bucket_count(const fftso3_batch* b) { return b ? (int)b->buckets.size() : -1; }

int fftso3_batch_stream_count(const fftso3_batch* b) { return b ? b->nstreams_used : -1; }

int fftso3_batch_graph_kernels(const fftso3_batch* b, int direction)
{
    if (!b || direction < 0 || direction > 1) return -1;
    return b->graphs[direction].exec ? b->graphs[direction].kernels : -1;
}

long long fftso3_batch_device_bytes(const fftso3_batch* b) { return b ? b->bytes : -1; }

int fftso3_batch_forward(fftso3_batch* b, const void* grids, void* coeffs, void* stream)
{
    return run(b, 0, grids, coeffs, stream);
}

int fftso3_batch_inverse(fftso3_batch* b, const void* coeffs, void* grids, void* stream)
{
    return run(b, 1, coeffs, grids, stream);
}

int fftso3_batch_bucket_info(const fftso3_batch* b, int bucket, int* l_max, int* count)
{
    if (!b || bucket < 0 || bucket >= (int)b->buckets.size())
        return bfail(FFTSO3_ERR_INVALID_ARG, "bucket index out of range");
    if (l_max) *l_max = b->buckets[bucket].L;
    if (count) *count = b->buckets[bucket].count;
    return FFTSO3_SUCCESS;
}

int fftso3_batch_set_timing(fftso3_batch* b, int enable)
{
    int rc = check_batch(b);
    if (rc) return rc;
    for (auto& k : b->buckets)
        if ((rc = fftso3_plan_set_timing(k.plan, enable))) return rc;
    b->timing = enable != 0;
    b->timer.enabled = enable != 0;
    return FFTSO3_SUCCESS;
}

int fftso3_batch_stage_times(fftso3_batch* b, int bucket, double* ms_total, long long* launches, int reset)
{
    int rc = check_batch(b);
    if (rc) return rc;
    if (bucket < -1 || bucket >= (int)b->buckets.size())
        return bfail(FFTSO3_ERR_INVALID_ARG, "bucket index out of range");
    const int ns = fftso3_stage_count();
    std::vector<double> ms(ns);
    std::vector<long long> cnt(ns);
    if (ms_total) std::fill(ms_total, ms_total + ns, 0.0);
    if (launches) std::fill(launches, launches + ns, 0LL);
    for (int i = 0; i < (int)b->buckets.size(); ++i) {
        if (bucket >= 0 && i != bucket) continue;
        if ((rc = fftso3_plan_stage_times(b->buckets[i].plan, ms.data(), cnt.data(), reset))) return rc;
        for (int s = 0; s < ns; ++s) {
            if (ms_total) ms_total[s] += ms[s];
            if (launches) launches[s] += cnt[s];
        }
    }
    if (bucket == -1) {  // the fused GEMM launches belong to no single bucket
        b->timer.collect();
        for (int s = 0; s < ns; ++s) {
            if (ms_total) ms_total[s] += b->timer.total_ms[s];
            if (launches) launches[s] += b->timer.launches[s];
        }
        if (reset) b->timer.reset();
    }
    return FFTSO3_SUCCESS;
}

int fftso3_batch_check(fftso3_batch* b)
{
    int rc = check_batch(b);
    if (rc) return rc;
    for (auto& k : b->buckets)
        if ((rc = fftso3_plan_check(k.plan))) return rc;
    if (b->fused) {
        const int code = tc_fused_status(b->fused);
        if (code != 0)
            return bfail(FFTSO3_ERR_CUDA,
                         "the fused tensor-core GEMM gave up a bounded wait (code " + std::to_string(code) + ")");
    }
    return FFTSO3_SUCCESS;
}

}  // extern "C"
