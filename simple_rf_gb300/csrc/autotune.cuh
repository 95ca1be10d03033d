// Online tile-shape tuning.  A launch site with several equivalent kernel shapes
// (same results, different speed) asks pick() for one: the first call with a new
// shape key times every candidate on the call's own inputs (CUDA events on the
// caller's stream, after one warm-up run each) and caches the fastest; later calls
// read the cache.  Only sites whose outputs are plain overwrites take part (a
// candidate that accumulates into its outputs would add twice), and nothing is
// timed while the stream is being captured into a CUDA graph or when tuning is
// off (srf_autotune_enable): those calls take the site's rule-of-thumb default.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace srf {
namespace tune {

enum Site : int {
    kSiteGemmEpilogueWarps = 1,   // tc_gemm_kernel: 8 or 4 epilogue warps (key: BN, K blocks, epilogue flags)
    kSiteBasisEncode = 2,         // basis_encode_kernel: rows per thread x threads (key: C, k1p)
    kSiteVmColorGroup = 3,        // color_fwd_group_kernel: lanes per point (key: R0, R1, R2)
};

struct Key {
    int site;
    int64_t a, b, c;
};

bool enabled();
int lookup(const Key& k);   // cached choice, or -1
void store(const Key& k, int choice);

// run(i) launches candidate i on stream s and returns its status (non-zero: the
// candidate does not apply and is skipped).  Returns the chosen candidate index.
template <class Run>
int pick(const Key& key, int n_cand, int fallback, cudaStream_t s, Run&& run) {
    const int cached = lookup(key);
    if (cached >= 0 && cached < n_cand) return cached;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (!enabled() || n_cand < 2 || cudaStreamIsCapturing(s, &cs) != cudaSuccess ||
        cs != cudaStreamCaptureStatusNone)
        return fallback;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return fallback;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fallback;
    }
    int best = -1;
    float best_ms = 0.f;
    for (int i = 0; i < n_cand; ++i) {
        if (run(i) != 0) continue;   // warm-up (and applicability)
        cudaEventRecord(e0, s);
        int st = 0;
        for (int r = 0; r < 3 && !st; ++r) st = run(i);
        cudaEventRecord(e1, s);
        if (st || cudaEventSynchronize(e1) != cudaSuccess) continue;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) continue;
        if (best < 0 || ms < best_ms) {
            best = i;
            best_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best < 0) return fallback;
    store(key, best);
    return best;
}

}  // namespace tune
}  // namespace srf
