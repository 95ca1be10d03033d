// Status strings, CUDA error text, the launch counter and the device-side error flag.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "autotune.cuh"
#include "srf_common.cuh"

namespace {
__device__ int g_srf_flag = 0;
thread_local char g_last_error[256] = "no error";
}  // namespace

namespace srf {

static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_cuda_error(cudaError_t e) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
}

int* device_flag() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    static int* cache[64] = {nullptr};
    if (dev < 0 || dev >= 64) return nullptr;
    if (!cache[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_srf_flag) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        cache[dev] = static_cast<int*>(p);
    }
    return cache[dev];
}

namespace tune {
namespace {
std::mutex g_tune_mu;
std::map<std::tuple<int, int64_t, int64_t, int64_t>, int> g_tune_table;
std::atomic<int> g_tune_on{1};
}  // namespace

bool enabled() { return g_tune_on.load() != 0; }

int lookup(const Key& k) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_table.find(std::make_tuple(k.site, k.a, k.b, k.c));
    return it == g_tune_table.end() ? -1 : it->second;
}

void store(const Key& k, int choice) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_table[std::make_tuple(k.site, k.a, k.b, k.c)] = choice;
}

int count() {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    return int(g_tune_table.size());
}

bool entry(int i, Key* k, int* choice) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (i < 0 || i >= int(g_tune_table.size())) return false;
    auto it = g_tune_table.begin();
    std::advance(it, i);
    *k = Key{std::get<0>(it->first), std::get<1>(it->first), std::get<2>(it->first), std::get<3>(it->first)};
    *choice = it->second;
    return true;
}

void clear() {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_table.clear();
}

void set_enabled(int on) { g_tune_on.store(on ? 1 : 0); }
}  // namespace tune

}  // namespace srf

extern "C" int srf_autotune_enable(int on) {
    srf::tune::set_enabled(on);
    return SRF_OK;
}

extern "C" int srf_autotune_count(void) { return srf::tune::count(); }

extern "C" int srf_autotune_entry(int index, int* site, int64_t* a, int64_t* b, int64_t* c, int* choice) {
    if (!site || !a || !b || !c || !choice) return SRF_ERR_NULL;
    srf::tune::Key k{};
    if (!srf::tune::entry(index, &k, choice)) return SRF_ERR_SHAPE;
    *site = k.site;
    *a = k.a;
    *b = k.b;
    *c = k.c;
    return SRF_OK;
}

extern "C" int srf_autotune_set(int site, int64_t a, int64_t b, int64_t c, int choice) {
    if (choice < 0) return SRF_ERR_SHAPE;
    srf::tune::store(srf::tune::Key{site, a, b, c}, choice);
    return SRF_OK;
}

extern "C" int srf_autotune_clear(void) {
    srf::tune::clear();
    return SRF_OK;
}

extern "C" const char* srf_status_string(int status) {
    switch (status) {
        case SRF_OK: return "SRF_OK";
        case SRF_ERR_NULL: return "SRF_ERR_NULL: a required pointer is NULL";
        case SRF_ERR_SHAPE: return "SRF_ERR_SHAPE: a size is out of the supported range";
        case SRF_ERR_ALIGN: return "SRF_ERR_ALIGN: a pointer or stride breaks an alignment rule";
        case SRF_ERR_WORKSPACE: return "SRF_ERR_WORKSPACE: workspace too small";
        case SRF_ERR_CUDA: return "SRF_ERR_CUDA: a CUDA call failed";
        case SRF_ERR_TIMEOUT: return "SRF_ERR_TIMEOUT: a bounded device wait gave up";
        case SRF_ERR_RANGE: return "SRF_ERR_RANGE: a device-side index check failed";
        case SRF_ERR_UNSUPPORTED: return "SRF_ERR_UNSUPPORTED: configuration not supported";
        default: return "unknown srf status";
    }
}

extern "C" const char* srf_version(void) { return "srf_gb300 1.0 sm_103a"; }

extern "C" const char* srf_last_cuda_error(void) { return g_last_error; }

extern "C" int64_t srf_launch_count(void) { return srf::g_launches.load(); }

extern "C" int srf_stream_create(void** stream_out) {
    if (!stream_out) return SRF_ERR_NULL;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        srf::set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    *stream_out = st;
    return SRF_OK;
}

extern "C" int srf_stream_destroy(void* stream) {
    if (!stream) return SRF_ERR_NULL;
    cudaError_t e = cudaStreamDestroy(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        srf::set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    return SRF_OK;
}

extern "C" int srf_read_device_flag(int* flag_out, void* stream) {
    if (!flag_out) return SRF_ERR_NULL;
    int* f = srf::device_flag();
    if (!f) return SRF_ERR_CUDA;
    int host = 0;
    cudaStream_t s = srf::as_stream(stream);
    cudaError_t e = cudaMemcpyAsync(&host, f, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(f, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        srf::set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    *flag_out = host;
    return SRF_OK;
}

// ------------------------------------------------------ bandwidth probe ----
// Streams a buffer `passes` times with 16-byte loads (grid-stride, every block
// walks the whole buffer's share of its threads), reducing to one float per
// block so the loads cannot be dropped.  A buffer smaller than L2 measures the
// L2 read rate the VM gathers are bounded by; a larger one the HBM read rate.
namespace {
__global__ void __launch_bounds__(512) read_probe_kernel(const float4* __restrict__ buf, int64_t n4, int passes,
                                                         float* __restrict__ sink) {
    float acc = 0.f;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int p = 0; p < passes; ++p) {
        for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n4; i += stride) {
            float4 v = __ldcg(buf + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ float part[16];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) s += part[w];
        sink[blockIdx.x] = s;
    }
}
}  // namespace

extern "C" int srf_read_probe_blocks(void) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        return 0;
    return 4 * sms;
}

extern "C" int srf_read_probe(const void* buf, int64_t bytes, int passes, float* sink, void* stream) {
    if (!buf || !sink) return SRF_ERR_NULL;
    if (bytes < 16 || (bytes & 15) || passes < 1 || (reinterpret_cast<uintptr_t>(buf) & 15)) return SRF_ERR_SHAPE;
    int blocks = srf_read_probe_blocks();
    if (blocks <= 0) return SRF_ERR_CUDA;
    read_probe_kernel<<<blocks, 512, 0, srf::as_stream(stream)>>>(static_cast<const float4*>(buf), bytes / 16, passes,
                                                                   sink);
    return srf::launch_status();
}
