// Library runtime: error reporting, setup, per-device scratch and the cached
// Student-t critical-value tables. Host code only.
#include <cuda.h>
#include <cuda_runtime.h>

#include <sys/mman.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>
#include <map>
#include <mutex>
#include <string>
#include <algorithm>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "tma_common.cuh"
#include "tquantile.h"

namespace stater {

void noalloc_forget_device(int dev);  // target_spp.cu
void df_tables_release(int dev);      // denoise_fast.cu

namespace {
thread_local std::string g_last_error;

struct ScratchBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct LutEntry {
    float *f32 = nullptr;
    double *f64 = nullptr;
};

std::mutex g_mutex;
std::map<std::tuple<int, cudaStream_t, int>, ScratchBuf> g_scratch;
std::map<std::pair<int, double>, LutEntry> g_luts;
std::map<int, int> g_sm_count;
std::map<int, int *> g_err_word;

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;

// Pipeline-wait settings of the TMA-fed kernels (stater_debug_set_pipeline_waits).
std::atomic<uint32_t> g_wait_limit{tma::kWaitLimit};
std::atomic<int> g_stall{0};
constexpr uint32_t kStallMaxPolls = 1u << 16;

constexpr int kLutIntervals = 1024;
}  // namespace

stater_status set_error(stater_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}

stater_status clear_error() {
    g_last_error.clear();
    return STATER_OK;
}

stater_status cuda_status(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return STATER_OK;
    return set_error(e == cudaErrorMemoryAllocation ? STATER_ERR_NOMEM : STATER_ERR_CUDA,
                     std::string(what) + ": " + cudaGetErrorString(e));
}

int sm_count() {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_mutex);
    auto it = g_sm_count.find(dev);
    if (it != g_sm_count.end()) return it->second;
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
    g_sm_count[dev] = n;
    return n;
}

void *scratch(int slot, size_t bytes, cudaStream_t stream) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_mutex);
    ScratchBuf &b = g_scratch[std::make_tuple(dev, stream, slot)];
    if (b.bytes >= bytes && b.ptr) return b.ptr;
    if (b.ptr) {
        // Earlier work on this stream may still read the old buffer.
        cudaStreamSynchronize(stream);
        cudaFree(b.ptr);
        b.ptr = nullptr;
        b.bytes = 0;
    }
    size_t want = bytes < 256 ? 256 : bytes;
    if (cudaMalloc(&b.ptr, want) != cudaSuccess) {
        cudaGetLastError();
        b.ptr = nullptr;
        return nullptr;
    }
    b.bytes = want;
    return b.ptr;
}

int tcrit_intervals() { return kLutIntervals; }

uint32_t pipeline_wait_limit() { return g_wait_limit.load(); }
int pipeline_stall() { return g_stall.load(); }

// One int per device that kernels set when a bounded wait gives up.
int *device_error_word() {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_mutex);
    int *&w = g_err_word[dev];
    if (!w) {
        if (cudaMalloc(&w, sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            w = nullptr;
            return nullptr;
        }
        cudaMemset(w, 0, sizeof(int));
    }
    return w;
}

// 2-D fp32 tensor map over a row-major [rows][cols] array (cols contiguous),
// boxes of box_rows x box_cols, out-of-range elements read as zero.
bool encode_tensor_map_2d_f32(CUtensorMap *map, const void *base, uint64_t cols, uint64_t rows, uint32_t box_cols,
                              uint32_t box_rows) {
    {
        std::lock_guard<std::mutex> lk(g_mutex);
        if (!g_encode) {
            void *fn = nullptr;
            cudaDriverEntryPointQueryResult q;
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                    cudaSuccess ||
                q != cudaDriverEntryPointSuccess || !fn) {
                cudaGetLastError();
                return false;
            }
            g_encode = (EncodeTiledFn)fn;
        }
    }
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 4};
    const cuuint32_t box[2] = {box_cols, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_tensor_map_3d_f32(CUtensorMap *map, const void *base, uint64_t d0, uint64_t d1, uint64_t d2, uint32_t b0,
                              uint32_t b1, uint32_t b2) {
    CUtensorMap probe;
    if (!encode_tensor_map_2d_f32(&probe, base, d0, d1 * d2, b0, 1)) return false;  // resolves the entry point
    const cuuint64_t dims[3] = {d0, d1, d2};
    const cuuint64_t strides[2] = {d0 * 4, d0 * d1 * 4};
    const cuuint32_t box[3] = {b0, b1, b2};
    const cuuint32_t estr[3] = {1, 1, 1};
    return g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

const void *tcrit_table_device(double alpha, bool f64, cudaStream_t stream) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_mutex);
    LutEntry &e = g_luts[std::make_pair(dev, alpha)];
    if (!e.f64) {
        std::vector<double> t(kLutIntervals + 1);
        tcrit2_table(alpha, kLutIntervals, t.data());
        std::vector<float> tf(t.begin(), t.end());
        if (cudaMalloc(&e.f64, sizeof(double) * t.size()) != cudaSuccess ||
            cudaMalloc(&e.f32, sizeof(float) * t.size()) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        cudaMemcpy(e.f64, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(e.f32, tf.data(), sizeof(float) * tf.size(), cudaMemcpyHostToDevice);
    }
    (void)stream;
    return f64 ? (const void *)e.f64 : (const void *)e.f32;
}

}  // namespace stater

using namespace stater;

extern "C" {

const char *stater_last_error(void) { return g_last_error.c_str(); }

int32_t stater_abi_version(void) { return STATER_ABI_VERSION; }

stater_status stater_setup(void) {
    clear_error();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetDeviceProperties");
    if (prop.major != 10 || prop.minor != 3)
        return set_error(STATER_ERR_UNSUPPORTED,
                         "libstater is built for sm_103a; device reports sm_" +
                             std::to_string(prop.major) + std::to_string(prop.minor));
    sm_count();
    return STATER_OK;
}

stater_status stater_synchronize(stater_stream stream) {
    clear_error();
    stater_status st = cuda_status(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize");
    if (st != STATER_OK) return st;
    int *w = nullptr;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        std::lock_guard<std::mutex> lk(g_mutex);
        auto it = g_err_word.find(dev);
        if (it != g_err_word.end()) w = it->second;
    }
    if (w) {
        int v = 0;
        cudaError_t e = cudaMemcpy(&v, w, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_status(e, "stater_synchronize: error word");
        if (v != 0) {
            cudaMemset(w, 0, sizeof(int));
            if (v & tma::kErrDrain)
                return set_error(STATER_ERR_TIMEOUT,
                                 "a bounded device wait gave up and so did the final wait for the copies in flight: "
                                 "the pipeline is lost and the affected call's results are undefined");
            return set_error(STATER_ERR_TIMEOUT, "a bounded device wait gave up (pipeline stalled); results of the "
                                                 "affected call are incomplete");
        }
    }
    return STATER_OK;
}

void stater_print_macro_configuration(void) {
    std::printf("==== stater runtime configuration ====\n");
    std::printf("ABI_VERSION = %d\n", STATER_ABI_VERSION);
    std::printf("MAX_TRANSFORMS = %d\n", STATER_MAX_TRANSFORMS);
    std::printf("MAX_GBUFFERS = %d\n", STATER_MAX_GBUFFERS);
    std::printf("MAX_RADIUS = %d\n", STATER_MAX_RADIUS);
    std::printf("TCRIT_LUT_INTERVALS = %d\n", kLutIntervals);
    std::printf("FULL_MULTI_TRANSFORM = per call (n_transforms 1..%d, Box-Cox lambdas or named transforms)\n",
                STATER_MAX_TRANSFORMS);
    std::printf("FILM_MULTI_TRANSFORM_MODE = per call (mt_mode: 2 = all transforms, 3 = Jarque-Bera select)\n");
    std::printf("USE_LEVC = per call (use_levc: 1 = LEV-corrected varCD / m2C)\n");
    std::printf("CASCADE_MODE = per call (discr_source: 0 = denoised variance [CASCADE_MODE=1], "
                "1 = sample variance [CASCADE_MODE=0])\n");
    std::printf("AS_MODE = per call (stater_calc_target_spp_ex as_source: 0 = ASM denoised varD, "
                "1 = ASN sample variance)\n");
    std::printf("variants: MCL = cascade + LEV (default); MC = cascade; M = neither; ASN+MCL = as_source 1; "
                "MT-JB = mt_mode 3\n");
    std::printf("PRECISION = per call (F64 plain form, F32 form)\n");
    std::printf("==== end ====\n");
}

stater_status stater_release_cache(void) {
    clear_error();
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceSynchronize();
    std::lock_guard<std::mutex> lk(g_mutex);
    for (auto it = g_scratch.begin(); it != g_scratch.end();) {
        if (std::get<0>(it->first) == dev) {
            cudaFree(it->second.ptr);
            it = g_scratch.erase(it);
        } else {
            ++it;
        }
    }
    {
        auto it = g_err_word.find(dev);
        if (it != g_err_word.end()) {
            cudaFree(it->second);
            g_err_word.erase(it);
        }
    }
    for (auto it = g_luts.begin(); it != g_luts.end();) {
        if (it->first.first == dev) {
            cudaFree(it->second.f32);
            cudaFree(it->second.f64);
            it = g_luts.erase(it);
        } else {
            ++it;
        }
    }
    noalloc_forget_device(dev);
    df_tables_release(dev);
    return STATER_OK;
}

stater_status stater_debug_set_pipeline_waits(uint32_t wait_polls, int32_t stall_producers) {
    clear_error();
    const uint32_t limit = wait_polls == 0 ? tma::kWaitLimit : wait_polls;
    if (limit > tma::kWaitLimit)
        return set_error(STATER_ERR_INVALID, "stater_debug_set_pipeline_waits: more polls than the default limit");
    if (stall_producers != 0 && stall_producers != 1)
        return set_error(STATER_ERR_INVALID, "stater_debug_set_pipeline_waits: stall_producers must be 0 or 1");
    if (stall_producers && limit > kStallMaxPolls)
        return set_error(STATER_ERR_INVALID, "stater_debug_set_pipeline_waits: a stall needs a wait limit of at most "
                                             "65536 polls");
    g_wait_limit.store(limit);
    g_stall.store(stall_producers);
    return STATER_OK;
}

// Page-locked host memory on huge pages. A renderer hands the library tens of
// GB of samples per image; the GPU reads host memory through address
// translations of the host's pages, and with base pages (4 or 64 KB) copies of
// such a buffer ran between 65 and 210 GB/s from one run to the next on the
// same GB300 host, while the same copies from huge pages (2 MB or 512 MB, as
// the kernel offers) held 210 GB/s. The memory is mapped anonymously, marked
// MADV_HUGEPAGE, touched by several threads (so the pages are allocated in
// parallel) and registered with CUDA; where the kernel offers no transparent
// huge pages it is still page-locked, on base pages.
stater_status stater_host_alloc(size_t bytes, void **out) {
    clear_error();
    if (!out || bytes == 0) return set_error(STATER_ERR_INVALID, "stater_host_alloc: bad arguments");
    *out = nullptr;
    void *p = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (p == MAP_FAILED) return set_error(STATER_ERR_NOMEM, "stater_host_alloc: mmap failed");
#ifdef MADV_HUGEPAGE
    madvise(p, bytes, MADV_HUGEPAGE);
#endif
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    const size_t part = (bytes + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++)
        th.emplace_back([=] {
            const size_t b0 = std::min(bytes, (size_t)t * part), b1 = std::min(bytes, b0 + part);
            if (b1 > b0) std::memset((char *)p + b0, 0, b1 - b0);
        });
    for (auto &x : th) x.join();
    cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
        munmap(p, bytes);
        return cuda_status(e, "stater_host_alloc: cudaHostRegister");
    }
    *out = p;
    return STATER_OK;
}

stater_status stater_host_free(void *ptr, size_t bytes) {
    clear_error();
    if (!ptr) return STATER_OK;
    cudaError_t e = cudaHostUnregister(ptr);
    munmap(ptr, bytes);
    return cuda_status(e, "stater_host_free: cudaHostUnregister");
}

int32_t stater_tcrit_lut_intervals(void) { return kLutIntervals; }

stater_status stater_tcrit2_table(double alpha, double *table) {
    clear_error();
    if (!(alpha > 0.0 && alpha < 1.0) || !table)
        return set_error(STATER_ERR_INVALID, "stater_tcrit2_table: alpha must be in (0, 1)");
    tcrit2_table(alpha, kLutIntervals, table);
    return STATER_OK;
}

double stater_t_quantile(double p, double df) { return t_quantile(p, df); }

}  // extern "C"
