// noalloc.cu -- exact k-NN search that allocates no device memory.
//
// Who needs this.  Some callers cannot call cudaMalloc: an application whose
// own allocator already owns the GPU's memory (a framework's caching pool that
// reserves the device up front, so a second allocator would fail or fragment
// it), and request paths that must not allocate because cudaMalloc can
// synchronise the device and stall for milliseconds.  ssg_knn_noalloc serves
// them: the caller passes the database, the queries and the result buffers
// (all in device memory), and the only scratch the search needs -- the
// candidate keys that the scan kernel hands to the merge kernel -- lives in a
// fixed array compiled into this library.
//
// The array.  g_noalloc_keys is a file-scope __device__ array of
// kNoAllocKeys 64-bit keys (16 MiB).  Every GPU that loads the library holds
// it until the process exits.  With lazy module loading (the CUDA default) the
// array is reserved by the first call into this library on a device, whatever
// that call is: a caller whose own pool will reserve the whole GPU should make
// one small call first (an m = 1 search, say) so that the reservation happens
// before its pool takes the memory.  Host code cannot use the array's name as
// a device address (on the host it only names a stand-in), so each call
// resolves the real address with cudaGetSymbolAddress while the device is
// current.  The lookup allocates nothing once the module is loaded; during a
// stream capture the address cached by an earlier call on the device is used
// instead (a capture must not load modules), so the first call on a device
// should come before any stream capture.  Nothing in the array has to start
// at zero: the scan writes every key slot the merge later reads.  All calls
// share the one array and leave the last call's keys in it, so calls whose
// work overlaps on the GPU (different streams, or several host threads
// without ordering) race; calls issued in order on one stream do not.
#include "ssgpu.h"
#include "common.cuh"
#include "kernels.h"

#include <algorithm>
#include <cstdio>
#include <mutex>

namespace {

constexpr int64_t kNoAllocKeys = int64_t(2) << 20;  // 2,097,152 keys = 16 MiB

static __device__ __align__(256) uint64_t g_noalloc_keys[kNoAllocKeys];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_keys_addr[kMaxDevices] = {nullptr};

int fail(int code, const char *fmt, long long a = 0, long long b = 0) {
    char buf[512];
    snprintf(buf, sizeof buf, fmt, a, b);
    return ssg::report_error(code, buf);
}

// Device address of g_noalloc_keys on the current device.  Outside a stream
// capture it is looked up on every call (so a device reset, which unloads
// the module, never leaves a stale address behind); while `st` is capturing
// the address cached by the last uncaptured call on this device is used.
int keys_for_current_device(cudaStream_t st, uint64_t **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SSG_ECUDA, "no current CUDA device");
    if (dev < 0 || dev >= kMaxDevices) return fail(SSG_EUNSUPPORTED, "device ordinal %lld out of range", dev);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(SSG_ECUDA, "querying the stream's capture status failed");
    }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_keys);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(SSG_ECUDA, "resolving the scratch array's device address failed");
        }
        g_keys_addr[dev] = p;
    } else if (!g_keys_addr[dev]) {
        return fail(SSG_EINVAL, "the first no-allocation search on a device must not be captured: "
                                "make one call before capturing");
    }
    *out = static_cast<uint64_t *>(g_keys_addr[dev]);
    return SSG_OK;
}

bool aligned(const void *p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

}  // namespace

extern "C" int ssg_knn_noalloc(int metric, const void *dev_db, int64_t dim, int64_t n, const void *dev_q, int64_t m,
                               int32_t k, uint32_t *dev_ids, float *dev_dists, void *stream) {
    if (metric == SSG_METRIC_COSINE)
        return fail(SSG_EUNSUPPORTED, "the no-allocation search supports SqL2, L2, NormCosine, InnerProduct and "
                                      "Hamming (Cosine needs per-row norms, i.e. more scratch)");
    if (metric < SSG_METRIC_SQL2 || metric > SSG_METRIC_HAMMING) return fail(SSG_EUNSUPPORTED, "unknown metric %lld", metric);
    if (!dev_db || !dev_q || !dev_ids || !dev_dists) return fail(SSG_EINVAL, "NULL device pointer");
    // the scans read Float32 rows element by element and sketches word by
    // word: misaligned buffers are refused here instead of faulting on the GPU
    const uintptr_t row_align = metric == SSG_METRIC_HAMMING ? 8 : 4;
    if (!aligned(dev_db, row_align) || !aligned(dev_q, row_align))
        return fail(SSG_EINVAL, "database and query buffers must be %lld-byte aligned", (long long)row_align);
    if (!aligned(dev_ids, 4) || !aligned(dev_dists, 4))
        return fail(SSG_EINVAL, "result buffers must be 4-byte aligned");
    if (dim <= 0 || n <= 0 || m <= 0 || k <= 0)
        return fail(SSG_EINVAL, "dim, n, m and k must be positive");
    if (metric == SSG_METRIC_HAMMING && dim > 32)
        return fail(SSG_EUNSUPPORTED, "Hamming sketches are limited to 32 words, got %lld", dim);
    if (n >= (int64_t(1) << 32) - 1) return fail(SSG_EINVAL, "database length %lld out of range", n);
    const int kk = int(std::min<int64_t>(k, n));
    if (int64_t(m) * kk > kNoAllocKeys)
        return fail(SSG_EINVAL,
                    "m * min(k, n) = %lld candidate keys exceed the fixed scratch of %lld keys (16 MiB); "
                    "split the query batch",
                    (long long)(int64_t(m) * kk), (long long)kNoAllocKeys);

    // splits: fill the GPU, keep splits long, stay inside the fixed scratch
    const int64_t qtiles = (m + 127) / 128;
    int64_t splits = (int64_t(4) * ssg::device_sm_count() + qtiles - 1) / qtiles;
    splits = std::min<int64_t>(splits, std::max<int64_t>(1, n / std::max<int64_t>(1024, int64_t(8) * kk)));
    splits = std::min<int64_t>(splits, std::max<int64_t>(1, 8192 / kk));
    splits = std::min<int64_t>(splits, kNoAllocKeys / (int64_t(m) * kk));
    splits = std::max<int64_t>(1, splits);

    ssg::ScanArgs a{};
    a.metric = metric;
    a.n = n;
    a.dim = dim;
    a.m = m;
    a.kk = kk;
    a.splits = int(splits);
    a.split_len = (n + splits - 1) / splits;
    a.id_base = 0;
    const size_t gheap = metric == SSG_METRIC_HAMMING ? ssg::hamming_gheap_bytes(a) : ssg::direct_gheap_bytes(a);
    if (gheap != 0)
        return fail(SSG_EUNSUPPORTED, "k = %lld needs more top-k storage than shared memory holds "
                                      "(the no-allocation search keeps its heaps on chip)", k);

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint64_t *keys = nullptr;
    int rc = keys_for_current_device(st, &keys);
    if (rc) return rc;
    a.cand = keys;

    cudaError_t e;
    if (metric == SSG_METRIC_HAMMING)
        e = ssg::launch_hamming(a, static_cast<const uint64_t *>(dev_db), static_cast<const uint64_t *>(dev_q), st,
                                nullptr);
    else
        e = ssg::launch_direct_f32(a, static_cast<const float *>(dev_db), nullptr, static_cast<const float *>(dev_q),
                                   nullptr, st, nullptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(SSG_ECUDA, "launching the scan kernel failed");
    }
    ssg::FinalizeArgs f{};
    f.cand = keys;
    f.segs = int(splits);
    f.kk = kk;
    f.m = m;
    f.k_out = k;
    f.exclude_self = 0;
    f.out_ids = dev_ids;
    f.out_dists = dev_dists;
    e = ssg::launch_finalize(f, st, nullptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(SSG_ECUDA, "launching the merge kernel failed");
    }
    return SSG_OK;
}
