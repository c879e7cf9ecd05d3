// noalloc.cu -- connected-component labelling for callers that must not allocate.
//
// Some host programs own all device memory themselves: a framework with its own
// caching allocator, or a service that reserves its whole memory budget at start-up,
// will not let a library call cudaMalloc / cudaFree (which also synchronise the device).
// hdog_ccl_noalloc serves them: the caller passes the mask and the label array, and the
// labelling's scratch -- the cross-tile edge list, its counter, the root bitmap and the
// status word -- lives in one file-scope device array of fixed size, below.
//
// That array exists once per device for as long as the library is loaded, and every
// call shares it: a call clears the parts that must start at zero and overwrites the
// rest, so consecutive calls on one stream are independent, but calls that overlap on
// the GPU (two streams, or two host threads) race on it.
#include <mutex>

#include "kernels.cuh"

namespace hdog {

// Largest volume hdog_ccl_noalloc accepts: 2^22 voxels (for example 256 x 256 x 64).
constexpr int64_t kNoAllocMaxVoxels = (int64_t)1 << 22;
constexpr int64_t kNoAllocEdges = kNoAllocMaxVoxels / 8 + 1024;
constexpr int64_t kNoAllocBlocks = kNoAllocMaxVoxels / kScanBlock;

// Scratch layout, byte offsets (each part 256-byte aligned).
constexpr size_t kNaSub = 0;                                              // Sub
constexpr size_t kNaStatus = 256;                                         // int
constexpr size_t kNaEdgeCount = 512;                                      // unsigned long long
constexpr size_t kNaBlkCounts = 768;                                      // uint32 per 4096 voxels
constexpr size_t kNaRootBits = kNaBlkCounts + ((kNoAllocBlocks * 4 + 255) / 256) * 256;
constexpr size_t kNaEdges = kNaRootBits + ((kNoAllocBlocks * (kScanBlock / 32) * 4 + 255) / 256) * 256;
constexpr size_t kNoAllocScratchBytes = kNaEdges + kNoAllocEdges * sizeof(int2);   // about 4.7 MB

static_assert(sizeof(Sub) <= kNaStatus, "descriptor slot too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch (in host code the array's name is only a host-side
// stand-in).  It is looked up with the device current, once per device context: the cache
// keeps the context's id (cuCtxGetId, unique for the life of the process), so after a
// cudaDeviceReset, which destroys the primary context and with it the module, the next
// call looks the address up again in the new context.
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);
constexpr int kMaxDevices = 64;
struct ScratchAddr {
  unsigned long long ctx_id = 0;
  void *addr = nullptr;
};
static ScratchAddr g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mu;

template <class F>
static F driver_fn(const char *name) {
  void *p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<F>(p);
}

// Id of the calling thread's current context, 0 when it cannot be read.
static unsigned long long current_ctx_id() {
  static CtxGetCurrentFn get_current = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
  static CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId");
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

static int scratch_for_current_device(unsigned char **out) {
  int dev = 0;
  HDOG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return hdog_set_cuda_error(cudaErrorInvalidDevice, "hdog_ccl_noalloc: device id");
  // makes the device's primary context current (created if need be), so its id can be read
  HDOG_CUDA_TRY(cudaSetDevice(dev));
  const unsigned long long id = current_ctx_id();
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  ScratchAddr &c = g_scratch_addr[dev];
  if (id == 0 || c.ctx_id != id || !c.addr) {
    void *p = nullptr;
    HDOG_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    c.addr = p;
    c.ctx_id = id;   // 0: the id was unreadable, so the next call looks the address up again
  }
  *out = static_cast<unsigned char *>(c.addr);
  return HDOG_OK;
}

}  // namespace hdog

using namespace hdog;

extern "C" int hdog_set_error(int code, const char *what);

extern "C" int hdog_ccl_noalloc(const uint8_t *d_mask, int32_t *d_labels, int width, int height, int depth,
                                void *stream) {
  if (!d_mask || !d_labels) return hdog_set_error(HDOG_ERR_ARG, "hdog_ccl_noalloc: null buffer");
  if (width < 2 || height < 2 || depth < 1)
    return hdog_set_error(HDOG_ERR_SHAPE, "hdog_ccl_noalloc: needs width, height >= 2 and depth >= 1");
  const int64_t n = (int64_t)width * height * depth;
  if (n > kNoAllocMaxVoxels)
    return hdog_set_error(HDOG_ERR_SHAPE, "hdog_ccl_noalloc: volume larger than its fixed scratch allows "
                                          "(2^22 voxels); use hdog_ccl with a context");
  unsigned char *base = nullptr;
  const int rc = scratch_for_current_device(&base);
  if (rc != HDOG_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  Sub S{};
  S.W = width; S.H = height; S.D = depth;
  S.depth_valid = depth;
  S.vox = 0;
  S.blk = 0;
  S.edge = 0;
  S.edge_cap = kNoAllocEdges;
  Sub *d_sub = reinterpret_cast<Sub *>(base + kNaSub);
  int *d_status = reinterpret_cast<int *>(base + kNaStatus);
  unsigned long long *d_edge_count = reinterpret_cast<unsigned long long *>(base + kNaEdgeCount);
  uint32_t *d_blk = reinterpret_cast<uint32_t *>(base + kNaBlkCounts);
  uint32_t *d_bits = reinterpret_cast<uint32_t *>(base + kNaRootBits);
  int2 *d_edges = reinterpret_cast<int2 *>(base + kNaEdges);
  int num_sms = 152, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  HDOG_CUDA_TRY(cudaMemcpyAsync(d_sub, &S, sizeof(Sub), cudaMemcpyHostToDevice, st));
  HDOG_CUDA_TRY(cudaMemsetAsync(d_status, 0, sizeof(int), st));   // the edge counter is cleared by launch_ccl
  launch_ccl(d_sub, 1, width, height, depth, n, d_mask, d_labels, d_edges, d_edge_count, d_bits, d_blk, d_status,
             num_sms, st);
  HDOG_CUDA_TRY(cudaGetLastError());
  int status = 0;
  HDOG_CUDA_TRY(cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  if (status) return hdog_set_error(status, "hdog_ccl_noalloc: a bounded device loop hit its limit");
  return HDOG_OK;
}
