// Per-stage CUDA-event timing of a plan's internal launches (enabled on demand).
#pragma once
#include <cuda_runtime.h>
#include <vector>

namespace fftso3 {

enum Stage {
    ST_FFT_ROWS = 0,
    ST_FFT_COLS,
    ST_NYQUIST,
    ST_FP64_FWD,
    ST_FP64_INV,
    ST_BASIS,
    ST_PACK_FWD,
    ST_GEMM_FWD,
    ST_PACK_INV,
    ST_GEMM_INV,
    ST_REFINE,
    ST_FFT_2D,
    ST_REF_CONTRACT,
    ST_REF_FFT,
    ST_FFT_SLICES,
    ST_CONVERT,
    ST_INV_CONTRACT,
    ST_INV_FFT,
    ST_COUNT
};

inline const char* stage_name(int s)
{
    static const char* names[ST_COUNT] = {"fft_rows", "fft_cols", "zero_nyquist", "fp64_fwd_contract",
                                          "fp64_inv_contract", "basis_convert", "tc_pack_fwd", "tc_gemm_fwd",
                                          "tc_pack_inv", "tc_gemm_inv", "tc_refine_elementwise", "fft_2d",
                                          "refine_exact_contract", "refine_fft_df32", "fft_slices",
                                          "coeff_convert", "exact_inverse_contract", "exact_inverse_fft_df32"};
    return (s >= 0 && s < ST_COUNT) ? names[s] : "";
}

struct StageTimer {
    bool enabled = false;
    std::vector<cudaEvent_t> pool;
    struct Rec {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    double total_ms[ST_COUNT] = {};
    long long launches[ST_COUNT] = {};
    int cur = -1;
    cudaEvent_t cur_a = nullptr;

    cudaEvent_t get()
    {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    void begin(int stage, cudaStream_t st)
    {
        if (!enabled) return;
        cur = stage;
        cur_a = get();
        cudaEventRecord(cur_a, st);
    }
    void end(cudaStream_t st)
    {
        if (!enabled || cur < 0) return;
        cudaEvent_t b = get();
        cudaEventRecord(b, st);
        recs.push_back({cur, cur_a, b});
        cur = -1;
    }
    // Waits for the recorded events and folds them into the totals.
    void collect()
    {
        for (auto& r : recs) {
            cudaEventSynchronize(r.b);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, r.a, r.b);
            total_ms[r.stage] += ms;
            launches[r.stage] += 1;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        recs.clear();
    }
    void reset()
    {
        collect();
        for (int i = 0; i < ST_COUNT; ++i) {
            total_ms[i] = 0.;
            launches[i] = 0;
        }
    }
    ~StageTimer()
    {
        for (auto& r : recs) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace fftso3
