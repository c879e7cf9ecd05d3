// capi.cu -- the C ABI of libhdog: contexts, stage entry points, the batched substack
// pipeline and the HDoG3D_main-compatible parameter-file runner.
//
// Reference host code this replaces: src/3D/HDoG3D_main.cpp (initializeGPU :58-109,
// processSubstack :134-257, main :260-319) and src/3D/utils.h (loadParamFile :95-157,
// loadImage :160-173, saveFeatureVector :204-250).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <future>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "json_min.hpp"
#include "kernels.cuh"

using namespace hdog;

namespace hdog {
thread_local KernelTimer *g_timer = nullptr;
}

// Per-kernel CUDA-event timing of a context (hdog_timing_enable / hdog_timing_read).
struct EventTimer : KernelTimer {
  struct Rec {
    const char *name;
    cudaEvent_t a, b;
  };
  std::vector<cudaEvent_t> pool;
  std::vector<Rec> pending;
  struct Acc {
    int64_t count = 0;
    double ms = 0.0;
  };
  std::vector<std::pair<std::string, Acc>> totals;
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  void begin(const char *name, cudaStream_t s) override {
    Rec r{name, get(), get()};
    cudaEventRecord(r.a, s);
    pending.push_back(r);
  }
  void end(cudaStream_t s) override {
    if (!pending.empty()) cudaEventRecord(pending.back().b, s);
  }
  // Host-side wall time of a phase of a call (names starting with "host_"), in milliseconds.
  void add_host(const char *name, double ms) {
    for (auto &t : totals)
      if (t.first == name) {
        t.second.count++;
        t.second.ms += ms;
        return;
      }
    totals.emplace_back(name, Acc());
    totals.back().second.count = 1;
    totals.back().second.ms = ms;
  }
  void collect() {
    for (Rec &r : pending) {
      cudaEventSynchronize(r.b);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.a, r.b);
      Acc *acc = nullptr;
      for (auto &t : totals)
        if (t.first == r.name) acc = &t.second;
      if (!acc) {
        totals.emplace_back(r.name, Acc());
        acc = &totals.back().second;
      }
      acc->count++;
      acc->ms += ms;
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    pending.clear();
  }
  ~EventTimer() override {
    for (Rec &r : pending) { pool.push_back(r.a); pool.push_back(r.b); }
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

static int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

extern "C" int hdog_set_cuda_error(cudaError_t e, const char *what) {
  return fail(HDOG_ERR_CUDA, std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) +
                                 ") in " + what);
}

extern "C" const char *hdog_last_error(void) { return g_last_error.c_str(); }
extern "C" int hdog_set_error(int code, const char *what) { return fail(code, what); }
extern "C" int hdog_abi_version(void) { return HDOG_ABI_VERSION; }

#define TRY(expr)                          \
  do {                                     \
    int rc__ = (expr);                     \
    if (rc__ != HDOG_OK) return rc__;      \
  } while (0)

// ------------------------------------------------------------------ parameters
// calcGaussianWeight (DoG3DFilter.cu:372-392), host side, same float/double steps.
static int gauss_taps(float sigma, float *h) {
  int lw = (int)(2.0 * sigma + 0.5);
  int length = lw * 2 + 1;
  float p, sum;
  sum = 1.f;
  h[lw] = 1.f;
  sigma *= sigma;
  for (int i = 1; i <= lw; i++) {
    p = (float)std::exp(-0.5 * i * i / sigma);
    h[lw - i] = p;
    h[lw + i] = p;
    sum += p * 2;
  }
  for (int i = 0; i < length; i++) h[i] /= sum;
  for (int i = length; i < kMaxTaps; i++) h[i] = 0;
  return lw;
}

extern "C" int hdog_gaussian_taps(float sigma, float *taps80, int *radius) {
  if (!taps80 || !radius) return fail(HDOG_ERR_ARG, "hdog_gaussian_taps: null pointer");
  if (!(sigma >= 0.0f) || (int)(2.0 * sigma + 0.5) * 2 + 1 > kMaxTaps)
    return fail(HDOG_ERR_SHAPE, "hdog_gaussian_taps: sigma must be in [0, 19.75)");
  *radius = gauss_taps(sigma, taps80);
  return HDOG_OK;
}

extern "C" int hdog_depth_margin(const hdog_params *p, int *margin) {
  if (!p || !margin) return fail(HDOG_ERR_ARG, "hdog_depth_margin: null pointer");
  float t[kMaxTaps];
  int r;
  TRY(hdog_gaussian_taps(p->sigma_z_large, t, &r));
  *margin = r + p->extra_depth_margin;
  return HDOG_OK;
}

static int validate(const hdog_params *p) {
  if (!p) return fail(HDOG_ERR_ARG, "null params");
  if (p->width < 2 || p->height < 2 || p->depth < 1)
    return fail(HDOG_ERR_SHAPE, "width and height must be >= 2 and depth >= 1");
  if ((int64_t)p->width * p->height * p->depth >= (int64_t)1 << 31)
    return fail(HDOG_ERR_SHAPE, "a substack must hold fewer than 2^31 voxels (labels are int32 voxel indices)");
  if (p->radius_norm_xy < 0 || p->radius_norm_z < 0 || p->radius_norm_xy > kMaxRadiusXY || p->radius_norm_z > 1000)
    return fail(HDOG_ERR_SHAPE, "radius_norm.xy_large must be in [0, 421] and z_large in [0, 1000]");
  if (p->erosion_radius_xy < 0 || p->erosion_radius_z < 0 || p->erosion_radius_xy > kMaxRadiusXY ||
      p->erosion_radius_z > 1000)
    return fail(HDOG_ERR_SHAPE, "erosion radius must be in [0, 421] (xy) and [0, 1000] (z)");
  float t[kMaxTaps];
  int r;
  const float sig[4] = {p->sigma_xy_small, p->sigma_z_small, p->sigma_xy_large, p->sigma_z_large};
  for (int k = 0; k < 4; k++) TRY(hdog_gaussian_taps(sig[k], t, &r));
  if (p->min_intensity < 0 || p->min_intensity > 65535) return fail(HDOG_ERR_ARG, "min_intensity must fit in uint16");
  if (p->min_size < 0 || p->min_size > 65535) return fail(HDOG_ERR_ARG, "min_size must fit in uint16");
  return HDOG_OK;
}

// ------------------------------------------------------------------ context
// Host copy of a call's records in page-locked memory, so that the device-to-host copies
// run at the link's speed; grows by doubling and keeps its size between calls.
struct RecordBuf {
  hdog_record *p = nullptr;
  size_t n = 0, cap = 0;
  bool reserve(size_t want) {
    if (want <= cap) return true;
    size_t nc = cap ? cap : (size_t)1 << 16;
    while (nc < want) nc *= 2;
    hdog_record *q = nullptr;
    if (cudaMallocHost(&q, nc * sizeof(hdog_record)) != cudaSuccess) return false;
    if (n) memcpy(q, p, n * sizeof(hdog_record));
    if (p) cudaFreeHost(p);
    p = q;
    cap = nc;
    return true;
  }
  void clear() { n = 0; }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = cap = 0;
  }
};

struct hdog_ctx {
  hdog_params p;
  int dev = 0;
  int max_sub = 0;
  int W = 0, H = 0, D = 0;
  int64_t nvox = 0;        // W*H*D
  int64_t reg_cap = 0;     // region slots per substack (background included)
  int64_t nblk = 0;        // per-substack block slots (voxel blocks and region blocks)
  int64_t nchk = 0;        // per-substack chunk slots
  int64_t edge_cap = 0;    // cross-tile CCL edges per substack
  int64_t fg_cap = 0;      // foreground-list entries per substack
  int num_sms = 152;
  int max_smem = 48 * 1024;
  bool use_sweep = true;   // fused DoG + Hessian sweep when the parameters allow it
  RecordBuf last;   // records of the last whole-chain call (hdog_last_records)
  RecordBuf aside;  // records of a host-input stack's last substack when it runs first
  int margin = 0;
  DogTaps taps;
  std::mutex mu;

  void *arena = nullptr;
  size_t arena_bytes = 0;
  uint16_t *img = nullptr;       // [max_sub * nvox] staging of host substacks
  float2 *fa = nullptr, *fb = nullptr;   // [max_sub * nvox] temps (min/max, box, DoG)
  float *norm = nullptr, *dog = nullptr;
  uint8_t *mask = nullptr;
  int32_t *labels = nullptr;
  uint32_t *root_bits = nullptr, *blk_counts = nullptr, *blk_offsets = nullptr, *chunk = nullptr;
  int2 *edges = nullptr;
  unsigned long long *edge_count = nullptr;
  FgEntry *fg = nullptr;
  unsigned long long *fg_count = nullptr;
  unsigned long long *fg_count_packed = nullptr;
  unsigned *qctr = nullptr;      // work-queue counters of the persistent sweeps
  LaunchShape shape;             // launch shape of the sweeps (autotuned per frame shape)
  bool tuned = false;            // shape and graph_batch chosen by the autotuner
  int graph_batch = 0;           // substacks per launch in the graph form (0: max_sub)
  std::string tune_report;       // JSON of the autotuner's timings
  RegionAcc acc{};
  RegionOut out{};
  hdog_record *records = nullptr;
  int64_t slots = 0;
  int64_t *num_regions = nullptr, *num_records = nullptr;
  int *status = nullptr;
  Sub *d_subs = nullptr;
  int64_t *d_seg = nullptr;      // [6][max_sub]: vseg off,len,chk ; rseg off,len,chk

  // pinned host staging
  Sub *h_subs = nullptr;
  int64_t *h_seg = nullptr;
  int64_t *h_counts = nullptr;   // [3*max_sub + 2]: records, regions, foreground counts per substack; status
  // device copy of a whole stack for hdog_run_stack with host input, copied in chunks on
  // copy_st (one event per batch) so that later chunks land while earlier batches run
  uint16_t *stack_buf = nullptr;
  size_t stack_bytes = 0;
  cudaStream_t copy_st = nullptr;
  std::vector<cudaEvent_t> chunk_ev;
  cudaEvent_t start_ev = nullptr;
  int host_batch = 1;   // substacks in the first batch of a host-input stack (0: max_sub)
  int64_t walk_limit = 0;   // HDOG_OPT_WALK_LIMIT (0: the substack's voxel count)
  EventTimer *timer = nullptr;
};

// Makes the context's kernel timer (if any) current on this thread for one API call.
struct TimerScope {
  explicit TimerScope(hdog_ctx *c) { g_timer = c->timer; }
  ~TimerScope() { g_timer = nullptr; }
};

// Wall time of a host phase of a call, added to the context's timing report when timing is on.
struct HostPhase {
  hdog_ctx *c;
  const char *name;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  HostPhase(hdog_ctx *c_, const char *n) : c(c_), name(n) {}
  ~HostPhase() {
    if (c->timer)
      c->timer->add_host(name, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
  }
};

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Layout {
  size_t off[48];
  int n = 0;
  size_t total = 0;
  size_t add(size_t bytes) {
    size_t o = total;
    off[n++] = o;
    total += align256(bytes);
    return o;
  }
};

static int64_t edge_capacity(int64_t nvox) { return nvox / 8 + 1024; }
static int64_t fg_capacity(int64_t nvox) { return nvox / 8 + 1024; }

static void plan(const hdog_params *p, int max_sub, int64_t &nvox, int64_t &reg_cap, int64_t &nblk,
                 int64_t &nchk, Layout &L) {
  nvox = (int64_t)p->width * p->height * p->depth;
  reg_cap = (int64_t)((p->width + 1) / 2) * ((p->height + 1) / 2) * ((p->depth + 1) / 2) + 1;
  const int64_t vb = (nvox + kScanBlock - 1) / kScanBlock, rb = (reg_cap + kFinalizeBlock - 1) / kFinalizeBlock;
  nblk = vb > rb ? vb : rb;
  nchk = (nblk + 1023) / 1024 + 1;
  const int64_t S = max_sub, slots = S * reg_cap;
  L.add(S * nvox * sizeof(uint16_t));        // 0 img
  L.add(S * nvox * sizeof(float2));          // 1 fa
  L.add(S * nvox * sizeof(float2));          // 2 fb
  L.add(S * nvox * sizeof(float));           // 3 norm
  L.add(S * nvox * sizeof(float));           // 4 dog
  L.add(S * nvox * sizeof(uint8_t));         // 5 mask
  L.add(S * nvox * sizeof(int32_t));         // 6 labels
  L.add(S * nblk * (kScanBlock / 32) * sizeof(uint32_t));   // 7 root bits
  L.add(S * nblk * sizeof(uint32_t));        // 8 blk counts
  L.add(S * nblk * sizeof(uint32_t));        // 9 blk offsets
  L.add(S * nchk * sizeof(uint32_t));        // 10 chunk
  L.add(slots * sizeof(int32_t));            // 11 acc.label
  L.add(slots * sizeof(uint32_t));           // 12 acc.count
  L.add(slots * sizeof(uint32_t));           // 13 acc.max_ord
  L.add(3 * slots * sizeof(unsigned long long));  // 14 acc.sum_xyz
  L.add(slots * sizeof(unsigned long long));      // 15 acc.sum_norm (fixed point)
  L.add(6 * slots * sizeof(unsigned long long));  // 16 acc.hess (fixed point)
  L.add(slots * sizeof(float));              // 17 out.intensity
  L.add(3 * slots * sizeof(float));          // 18 out.centroid
  L.add(6 * slots * sizeof(float));          // 19 out.hessian
  L.add(2 * slots * sizeof(float));          // 20 out.eigen
  L.add(slots * sizeof(uint8_t));            // 21 out.keep
  L.add(slots * sizeof(hdog_record));        // 22 records
  L.add(S * sizeof(int64_t));                // 23 num_regions
  L.add(S * sizeof(int64_t));                // 24 num_records
  L.add(sizeof(int));                        // 25 status
  L.add(S * sizeof(Sub));                    // 26 subs
  L.add(6 * S * sizeof(int64_t));            // 27 seg
  L.add(S * edge_capacity(nvox) * sizeof(int2));          // 28 cross-tile edges
  L.add(S * sizeof(unsigned long long));     // 29 edge counts
  L.add(S * fg_capacity(nvox) * sizeof(FgEntry));         // 30 foreground list
  L.add(S * kFgCountStride * sizeof(unsigned long long));   // 31 foreground counts (strided)
  L.add(S * sizeof(unsigned long long));     // 32 foreground counts, packed for the read-back
  L.add(4 * sizeof(unsigned));               // 33 work-queue counters
}

extern "C" int hdog_ctx_bytes(const hdog_params *p, int max_substacks, size_t *bytes) {
  TRY(validate(p));
  if (max_substacks < 1 || !bytes) return fail(HDOG_ERR_ARG, "hdog_ctx_bytes: bad arguments");
  int64_t nvox, reg_cap, nblk, nchk;
  Layout L;
  plan(p, max_substacks, nvox, reg_cap, nblk, nchk, L);
  *bytes = L.total;
  return HDOG_OK;
}

static int make_taps(const hdog_params *p, DogTaps &T) {
  memset(&T, 0, sizeof(T));
  const float sig[4] = {p->sigma_xy_small, p->sigma_z_small, p->sigma_xy_large, p->sigma_z_large};
  for (int k = 0; k < 4; k++) T.r[k] = gauss_taps(sig[k], T.k[k]);
  // DoG3DFilter.cu:432, host powf as in the reference
  T.normalizer = powf(p->sigma_xy_small, p->gamma_n * 2) * powf(p->sigma_z_small, p->gamma_n);
  return HDOG_OK;
}

extern "C" int hdog_ctx_destroy(hdog_ctx *ctx) {
  if (!ctx) return HDOG_OK;
  cudaSetDevice(ctx->dev);
  if (ctx->arena) cudaFree(ctx->arena);
  if (ctx->stack_buf) cudaFree(ctx->stack_buf);
  for (cudaEvent_t e : ctx->chunk_ev) cudaEventDestroy(e);
  if (ctx->start_ev) cudaEventDestroy(ctx->start_ev);
  if (ctx->copy_st) cudaStreamDestroy(ctx->copy_st);
  if (ctx->h_subs) cudaFreeHost(ctx->h_subs);
  ctx->last.release();
  ctx->aside.release();
  delete ctx->timer;
  delete ctx;
  return HDOG_OK;
}

extern "C" int hdog_ctx_create(const hdog_params *p, int max_substacks, hdog_ctx **out) {
  if (!out) return fail(HDOG_ERR_ARG, "hdog_ctx_create: null output pointer");
  *out = nullptr;
  TRY(validate(p));
  if (max_substacks < 1 || max_substacks > 65535) return fail(HDOG_ERR_ARG, "max_substacks must be in [1, 65535]");
  HDOG_CUDA_TRY(cudaSetDevice(p->dev_id));
  hdog_ctx *c = new hdog_ctx();
  c->p = *p;
  c->dev = p->dev_id;
  c->max_sub = max_substacks;
  c->W = p->width; c->H = p->height; c->D = p->depth;
  Layout L;
  plan(p, max_substacks, c->nvox, c->reg_cap, c->nblk, c->nchk, L);
  c->slots = (int64_t)max_substacks * c->reg_cap;
  TRY(hdog_depth_margin(p, &c->margin));
  make_taps(p, c->taps);
  cudaError_t e = cudaMalloc(&c->arena, L.total);
  if (e != cudaSuccess) {
    delete c;
    return fail(HDOG_ERR_NOMEM, "hdog_ctx_create: cudaMalloc of " + std::to_string(L.total) + " bytes failed");
  }
  c->arena_bytes = L.total;
  char *a = (char *)c->arena;
  auto at = [&](int i) { return (void *)(a + L.off[i]); };
  c->img = (uint16_t *)at(0);
  c->fa = (float2 *)at(1);
  c->fb = (float2 *)at(2);
  c->norm = (float *)at(3);
  c->dog = (float *)at(4);
  c->mask = (uint8_t *)at(5);
  c->labels = (int32_t *)at(6);
  c->root_bits = (uint32_t *)at(7);
  c->blk_counts = (uint32_t *)at(8);
  c->blk_offsets = (uint32_t *)at(9);
  c->chunk = (uint32_t *)at(10);
  c->acc.label = (int32_t *)at(11);
  c->acc.count = (uint32_t *)at(12);
  c->acc.max_ord = (uint32_t *)at(13);
  c->acc.sum_xyz = (unsigned long long *)at(14);
  c->acc.sum_norm = (unsigned long long *)at(15);
  c->acc.hess = (unsigned long long *)at(16);
  c->out.intensity = (float *)at(17);
  c->out.centroid = (float *)at(18);
  c->out.hessian = (float *)at(19);
  c->out.eigen = (float *)at(20);
  c->out.keep = (uint8_t *)at(21);
  c->records = (hdog_record *)at(22);
  c->num_regions = (int64_t *)at(23);
  c->num_records = (int64_t *)at(24);
  c->status = (int *)at(25);
  c->d_subs = (Sub *)at(26);
  c->d_seg = (int64_t *)at(27);
  c->edges = (int2 *)at(28);
  c->edge_count = (unsigned long long *)at(29);
  c->edge_cap = edge_capacity(c->nvox);
  c->fg = (FgEntry *)at(30);
  c->fg_count = (unsigned long long *)at(31);
  c->fg_count_packed = (unsigned long long *)at(32);
  c->fg_cap = fg_capacity(c->nvox);
  c->qctr = (unsigned *)at(33);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->dev);
  c->shape.num_sms = c->num_sms;
  cudaDeviceGetAttribute(&c->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->dev);
  const size_t hb = (size_t)max_substacks * sizeof(Sub) + 6 * (size_t)max_substacks * sizeof(int64_t) +
                    (3 * (size_t)max_substacks + 2) * sizeof(int64_t);
  e = cudaMallocHost(&c->h_subs, hb);
  if (e != cudaSuccess) {
    cudaFree(c->arena);
    delete c;
    return fail(HDOG_ERR_NOMEM, "hdog_ctx_create: pinned host staging failed");
  }
  c->h_seg = (int64_t *)(c->h_subs + max_substacks);
  c->h_counts = c->h_seg + 6 * max_substacks;
  *out = c;
  return HDOG_OK;
}

// ------------------------------------------------------------------ batch helpers
// all_eigen: eigen features for every region (the stage API returns them), else only
// for the regions that become records.
static FilterParams filter_of(const hdog_params &p, bool all_eigen = false) {
  FilterParams f;
  f.left = p.left_margin; f.right = p.right_margin; f.top = p.top_margin; f.bottom = p.bottom_margin;
  f.min_size = p.min_size;
  f.is_ave_mode = p.is_ave_mode;
  f.all_eigen = all_eigen ? 1 : 0;
  return f;
}

// Fills the host descriptors of substack s (not yet uploaded).
static void set_sub(hdog_ctx *c, int s, const uint16_t *src, int depth_valid, int z0) {
  Sub &S = c->h_subs[s];
  S.W = c->W; S.H = c->H; S.D = c->D;
  S.depth_valid = depth_valid;
  S.z0 = z0;
  S.margin = c->margin;
  S.vox = (int64_t)s * c->nvox;
  S.reg = (int64_t)s * c->reg_cap;
  S.reg_cap = c->reg_cap;
  S.blk = (int64_t)s * c->nblk;
  S.edge = (int64_t)s * c->edge_cap;
  S.edge_cap = c->edge_cap;
  S.fg = (int64_t)s * c->fg_cap;
  S.fg_cap = c->fg_cap;
  S.src = src;
  S.walk_limit = c->walk_limit;
  const int ms = c->max_sub;
  c->h_seg[0 * ms + s] = S.blk;
  c->h_seg[1 * ms + s] = (c->nvox + kScanBlock - 1) / kScanBlock;
  c->h_seg[2 * ms + s] = (int64_t)s * c->nchk;
  c->h_seg[3 * ms + s] = S.blk;
  c->h_seg[4 * ms + s] = (c->reg_cap + kFinalizeBlock - 1) / kFinalizeBlock;
  c->h_seg[5 * ms + s] = (int64_t)s * c->nchk;
}

// Whether every substack's input starts on an 8-byte boundary (vector loads of four
// uint16 in the z min/max pass).
static bool srcs_aligned8(const hdog_ctx *c, int nsub) {
  for (int s = 0; s < nsub; s++)
    if (reinterpret_cast<uintptr_t>(c->h_subs[s].src) & 7) return false;
  return true;
}

// The batch's descriptors travel as kernel parameters, kParamSubs substacks per launch, and a
// one-block kernel stores them: no host-to-device copy on the compute stream, where it would
// queue on the copy engine behind a stack chunk that hdog_run_stack is copying on its copy
// stream, and nothing that a captured graph would read from host memory at replay (a
// captured copy reads its source when the graph runs, by then the last batch's descriptors).
constexpr int kParamSubs = 16;
struct SubsParam {
  Sub subs[kParamSubs];
  int64_t seg[6][kParamSubs];
};

// substacks [s0, s0 + n) of the context's ms slots: the first nsub of them get descriptors,
// every slot its six scan-segment entries (seg is [6][ms])
__global__ void k_store_subs(const __grid_constant__ SubsParam P, int s0, int n, int nsub, int ms, Sub *subs,
                             int64_t *seg) {
  const int t = threadIdx.x;
  if (t < n && s0 + t < nsub) subs[s0 + t] = P.subs[t];
  if (t < 6 * n) seg[(int64_t)(t / n) * ms + s0 + t % n] = P.seg[t / n][t % n];
}

static int upload_subs(hdog_ctx *c, int nsub, cudaStream_t st) {
  const int ms = c->max_sub;
  for (int s0 = 0; s0 < ms; s0 += kParamSubs) {
    const int n = std::min(kParamSubs, ms - s0);
    SubsParam P;
    memset(&P, 0, sizeof(P));
    const int ns = std::max(0, std::min(n, nsub - s0));
    if (ns > 0) memcpy(P.subs, c->h_subs + s0, ns * sizeof(Sub));
    for (int k = 0; k < 6; k++) memcpy(P.seg[k], c->h_seg + (size_t)k * ms + s0, n * sizeof(int64_t));
    KLAUNCH("k_store_subs", st, (k_store_subs<<<1, 6 * kParamSubs, 0, st>>>(P, s0, n, nsub, ms, c->d_subs, c->d_seg)));
    HDOG_CUDA_TRY(cudaGetLastError());
  }
  return HDOG_OK;
}

static ScanSeg vseg_of(hdog_ctx *c) {
  const int ms = c->max_sub;
  return ScanSeg{c->d_seg, c->d_seg + ms, c->d_seg + 2 * ms, (c->nvox + kScanBlock - 1) / kScanBlock};
}
static ScanSeg rseg_of(hdog_ctx *c) {
  const int ms = c->max_sub;
  return ScanSeg{c->d_seg + 3 * ms, c->d_seg + 4 * ms, c->d_seg + 5 * ms,
                 (c->reg_cap + kFinalizeBlock - 1) / kFinalizeBlock};
}

// Normalization of nsub substacks (descriptors already uploaded): src -> out_norm, and
// the box means of the min and the max when ero_l / dil_l are given.
static void enqueue_normalize(hdog_ctx *c, int nsub, float *out_norm, cudaStream_t st, float *ero_l = nullptr,
                              float *dil_l = nullptr) {
  const hdog_params &p = c->p;
  if (p.radius_norm_xy == 0 || p.radius_norm_z == 0) {
    launch_copy_norm(c->d_subs, nsub, c->nvox, (float)p.min_intensity, out_norm, st);
    if (ero_l) {   // no box means on the copy path: zero planes
      zero_async(ero_l, (size_t)nsub * c->nvox * sizeof(float), st);
      zero_async(dil_l, (size_t)nsub * c->nvox * sizeof(float), st);
    }
    return;
  }
  // min/max (exact) z -> y -> x, box means x -> y -> z; packed u32 in fb's halves
  uint32_t *ma = reinterpret_cast<uint32_t *>(c->fb);
  uint32_t *mb = ma + (int64_t)c->max_sub * c->nvox;
  launch_normalize(c->d_subs, nsub, c->W, c->H, c->D, p.radius_norm_xy, p.radius_norm_z, (float)p.min_intensity,
                   srcs_aligned8(c, nsub), ma, mb, c->fa, c->fb, out_norm, st, ero_l, dil_l);
}

// DoG volume: the radius-specialised z-sweep where it applies (bit-identical), else the
// three separate passes.
static void enqueue_dog(hdog_ctx *c, int nsub, const float *norm, float *dog, cudaStream_t st) {
  if (c->use_sweep && launch_dog_sweep(c->d_subs, nsub, c->W, c->H, c->D, c->taps, norm, dog, c->status, c->max_smem, st))
    return;
  launch_dog(c->d_subs, nsub, c->W, c->H, c->D, (int64_t)c->H * c->D, c->taps, norm, c->fa, c->fb, dog, st);
}

// The chain after normalization: DoG + Hessian (fused sweep or separate passes), CCL,
// region numbering and accumulation, features and record compaction.
static void enqueue_after_norm(hdog_ctx *c, int nsub, bool fused, cudaStream_t st) {
  // each foreground entry's voxel index, then its root (written by the CCL flatten), per
  // entry beside the list (fb is free after the normalization)
  int32_t *fg_root = reinterpret_cast<int32_t *>(c->fb);
  if (fused) {
    launch_dog_hess(c->d_subs, nsub, c->W, c->H, c->D, c->taps, c->norm, c->dog, c->mask, c->fg, fg_root,
                    c->fg_count, c->status, c->shape, c->qctr, st);
  } else {
    enqueue_dog(c, nsub, c->norm, c->dog, st);
    launch_hessian_pd(c->d_subs, nsub, c->W, c->H, c->D, c->dog, c->mask, nullptr, st);
  }
  launch_ccl(c->d_subs, nsub, c->W, c->H, c->D, c->nvox, c->mask, c->labels, c->edges, c->edge_count, c->root_bits,
             c->blk_counts, c->status, c->num_sms, st, fused ? c->fg : nullptr, fused ? c->fg_count : nullptr,
             c->fg_cap, c->nblk, fg_root);
  int32_t *rank = reinterpret_cast<int32_t *>(c->fa);
  if (fused)
    launch_regions_fg(c->d_subs, nsub, c->nvox, c->fg_cap, vseg_of(c), fg_root, c->root_bits, c->fg, c->fg_count, rank,
                      c->blk_counts, c->blk_offsets, c->chunk, c->num_regions, c->acc, c->slots, c->status, c->num_sms,
                      st);
  else
    launch_regions(c->d_subs, nsub, c->nvox, vseg_of(c), c->mask, c->labels, c->root_bits, c->norm, c->dog, rank,
                   c->blk_counts, c->blk_offsets, c->chunk, c->num_regions, c->acc, c->slots, c->status, st);
  launch_finalize(c->d_subs, nsub, c->reg_cap, rseg_of(c), c->num_regions, c->acc, c->slots, c->out, filter_of(c->p),
                  c->blk_counts, c->blk_offsets, c->chunk, c->num_records, c->records, c->nblk, st);
}

// The fused sweep and the list-based region sums; the latter add coordinates in 32 bits
// inside a warp (at most 512 entries of coordinates below 2^16), so larger frames take
// the separate passes.
static bool fused_ok(hdog_ctx *c) {
  return c->use_sweep && c->W <= 65535 && c->H <= 65535 && c->D <= 65535 &&
         sweep_supported(c->taps, c->W, c->max_smem);
}

// Reads record / region / foreground counts and the status word back (one sync).
static int readback(hdog_ctx *c, int nsub, cudaStream_t st) {
  const int ms = c->max_sub;
  HDOG_CUDA_TRY(cudaGetLastError());
  HDOG_CUDA_TRY(cudaMemcpyAsync(c->h_counts, c->num_records, nsub * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  HDOG_CUDA_TRY(cudaMemcpyAsync(c->h_counts + ms, c->num_regions, nsub * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  // a strided (2D) copy could wait on the copy engine behind a host stack's chunks, so the
  // counters are packed on the device first
  pack_fg_counts_async(c->fg_count, nsub, c->fg_count_packed, st);
  HDOG_CUDA_TRY(cudaMemcpyAsync(c->h_counts + 2 * ms, c->fg_count_packed, nsub * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                st));
  HDOG_CUDA_TRY(cudaMemcpyAsync(c->h_counts + 3 * ms, c->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  const int status = *(int *)(c->h_counts + 3 * ms);
  if (status == HDOG_ERR_CAPACITY) return fail(HDOG_ERR_CAPACITY, "region capacity exceeded");
  if (status != 0) return fail(status, "a bounded device wait or loop hit its limit");
  return HDOG_OK;
}

// Whole chain for nsub substacks whose descriptors are set (host side).  Leaves record
// counts, region counts and the status word in c->h_counts after a stream sync.
// Enqueues the whole chain for nsub substacks whose host descriptors are set, up to the
// records in c->records (no host synchronization).
static int enqueue_batch(hdog_ctx *c, int nsub, bool fused, cudaStream_t st) {
  TRY(upload_subs(c, nsub, st));
  zero_async(c->status, sizeof(int), st);
  if (c->p.erosion_radius_xy > 0 || c->p.erosion_radius_z > 0) {
    // opt-in regional erosion of the input (the reference compiles Erosion3DFilter but
    // never calls it); the eroded substacks replace the inputs in c->img
    launch_erosion(c->d_subs, nsub, c->W, c->H, c->D, c->p.erosion_radius_xy, c->p.erosion_radius_z,
                   srcs_aligned8(c, nsub), reinterpret_cast<uint32_t *>(c->fa), c->img, st);
    for (int s = 0; s < nsub; s++) {
      c->h_subs[s].src = c->img + (int64_t)s * c->nvox;
      c->h_subs[s].depth_valid = c->D;   // the eroded volume already carries the zero tail
    }
    TRY(upload_subs(c, nsub, st));
  }
  enqueue_normalize(c, nsub, c->norm, st);
  if (fused) zero_async(c->fg_count, (size_t)nsub * kFgCountStride * sizeof(unsigned long long), st);
  enqueue_after_norm(c, nsub, fused, st);
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

static int run_batch(hdog_ctx *c, int nsub, cudaStream_t st) {
  nvtxRangePushA("hdog batch");
  struct Pop {
    ~Pop() { nvtxRangePop(); }
  } pop;
  const bool fused = fused_ok(c);
  {
    HostPhase ph(c, "host_enqueue_batch");
    TRY(enqueue_batch(c, nsub, fused, st));
  }
  {
    HostPhase ph(c, "host_wait_batch");
    TRY(readback(c, nsub, st));
  }
  if (fused) {
    bool over = false;
    for (int s = 0; s < nsub; s++) over |= c->h_counts[2 * c->max_sub + s] > c->fg_cap;
    if (over) {
      // more foreground than the list holds: redo this batch with the separate passes
      zero_async(c->status, sizeof(int), st);
      enqueue_after_norm(c, nsub, false, st);
      TRY(readback(c, nsub, st));
    }
  }
  return HDOG_OK;
}

// Appends the records of substacks [0, nsub) to out, in substack order.
// The batch's records appended to `out`; with `direct`, a page-locked caller buffer of
// `direct_cap` records, they are also copied to the same positions there while they fit.
static int collect_records(hdog_ctx *c, int nsub, RecordBuf &out, cudaStream_t st, hdog_record *direct = nullptr,
                           int64_t direct_cap = 0) {
  HostPhase ph(c, "host_collect_records");
  size_t n = out.n, total = n;
  for (int s = 0; s < nsub; s++) total += (size_t)c->h_counts[s];
  if (!out.reserve(total)) return fail(HDOG_ERR_NOMEM, "page-locked host buffer for the records failed");
  for (int s = 0; s < nsub; s++) {
    const int64_t k = c->h_counts[s];
    if (k > 0) {
      const hdog_record *src = c->records + (int64_t)s * c->reg_cap;
      HDOG_CUDA_TRY(cudaMemcpyAsync(out.p + n, src, k * sizeof(hdog_record), cudaMemcpyDeviceToHost, st));
      if (direct && (int64_t)n + k <= direct_cap)
        HDOG_CUDA_TRY(cudaMemcpyAsync(direct + n, src, k * sizeof(hdog_record), cudaMemcpyDeviceToHost, st));
    }
    n += (size_t)k;
  }
  HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  out.n = total;
  return HDOG_OK;
}

// Host-to-host copy split over up to eight threads of at least 4 MB each: one core moves
// about 25 GB/s, and a full stack's records are tens of MB.  A thread that cannot be
// started leaves its part to the calling thread.
static void host_copy(void *dst, const void *src, size_t bytes) {
  constexpr size_t kPart = (size_t)4 << 20;
  const size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min({(size_t)8, hw, bytes / kPart});
  if (nt <= 1) {
    memcpy(dst, src, bytes);
    return;
  }
  const size_t per = (bytes + nt - 1) / nt;
  auto part = [=](size_t i) {
    const size_t off = i * per;
    if (off < bytes)
      memcpy(static_cast<char *>(dst) + off, static_cast<const char *>(src) + off, std::min(per, bytes - off));
  };
  std::vector<std::thread> th;
  std::vector<size_t> left;
  for (size_t i = 1; i < nt; i++) {
    try {
      th.emplace_back(part, i);
    } catch (...) {
      left.push_back(i);
    }
  }
  part(0);
  for (size_t i : left) part(i);
  for (std::thread &t : th) t.join();
}

// Records gathered from `src` into `dst` piece by piece, piece k (src offset, count) landing
// after the pieces before it, split over up to eight threads of at least 4 MB each (a run's
// records are up to a few GB).  A thread that cannot be started leaves its part to the
// calling thread.
static void host_gather(hdog_record *dst, const hdog_record *src, const std::vector<std::pair<size_t, size_t>> &pieces,
                        size_t total) {
  constexpr size_t kPart = ((size_t)4 << 20) / sizeof(hdog_record);
  const size_t hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::max((size_t)1, std::min({(size_t)8, hw, total / kPart}));
  // thread i copies the records [i * per, (i + 1) * per) of the output, whichever pieces they fall in
  const size_t per = (total + nt - 1) / nt;
  std::vector<size_t> dst_off(pieces.size());
  for (size_t k = 0, o = 0; k < pieces.size(); k++) {
    dst_off[k] = o;
    o += pieces[k].second;
  }
  auto part = [&](size_t i) {
    const size_t a = i * per, b = std::min(total, a + per);
    if (a >= b) return;
    // first piece that ends after a
    size_t k = std::upper_bound(dst_off.begin(), dst_off.end(), a) - dst_off.begin();
    k = k ? k - 1 : 0;
    for (; k < pieces.size() && dst_off[k] < b; k++) {
      const size_t lo = std::max(a, dst_off[k]), hi = std::min(b, dst_off[k] + pieces[k].second);
      if (hi > lo) memcpy(dst + lo, src + pieces[k].first + (lo - dst_off[k]), (hi - lo) * sizeof(hdog_record));
    }
  };
  std::vector<std::thread> th;
  std::vector<size_t> left;
  for (size_t i = 1; i < nt; i++) {
    try {
      th.emplace_back(part, i);
    } catch (...) {
      left.push_back(i);
    }
  }
  part(0);
  for (size_t i : left) part(i);
  for (std::thread &t : th) t.join();
}

static int copy_out(const RecordBuf &v, hdog_record *out, int64_t cap, int64_t *n) {
  *n = (int64_t)v.n;
  if (*n > cap) return fail(HDOG_ERR_CAPACITY, "record buffer too small: " + std::to_string(*n) + " records");
  if (*n > 0) host_copy(out, v.p, v.n * sizeof(hdog_record));
  return HDOG_OK;
}

// ------------------------------------------------------------------ stage entry points
static int single_sub(hdog_ctx *c, const uint16_t *src, cudaStream_t st) {
  set_sub(c, 0, src, c->D, 0);
  return upload_subs(c, 1, st);
}

#define CTX_GUARD(c)                                                   \
  if (!(c)) return fail(HDOG_ERR_ARG, "null context");                 \
  std::lock_guard<std::mutex> lock__((c)->mu);                         \
  TimerScope timer_scope__(c);                                         \
  HDOG_CUDA_TRY(cudaSetDevice((c)->dev))

extern "C" int hdog_normalize(hdog_ctx *c, const uint16_t *d_img, float *d_norm, void *stream) {
  CTX_GUARD(c);
  if (!d_img || !d_norm) return fail(HDOG_ERR_ARG, "hdog_normalize: null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  TRY(single_sub(c, d_img, st));
  enqueue_normalize(c, 1, d_norm, st);
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

extern "C" int hdog_normalize_parts(hdog_ctx *c, const uint16_t *d_img, float *d_norm, float *d_ero_l, float *d_dil_l,
                                    void *stream) {
  CTX_GUARD(c);
  if (!d_img || !d_norm || !d_ero_l || !d_dil_l) return fail(HDOG_ERR_ARG, "hdog_normalize_parts: null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  TRY(single_sub(c, d_img, st));
  enqueue_normalize(c, 1, d_norm, st, d_ero_l, d_dil_l);
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

extern "C" int hdog_dog(hdog_ctx *c, const float *d_norm, float *d_dog, void *stream) {
  CTX_GUARD(c);
  if (!d_norm || !d_dog) return fail(HDOG_ERR_ARG, "hdog_dog: null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  TRY(single_sub(c, nullptr, st));
  zero_async(c->status, sizeof(int), st);
  enqueue_dog(c, 1, d_norm, d_dog, st);
  HDOG_CUDA_TRY(cudaGetLastError());
  // the sweep's bounded TMA waits report through the status word
  int status = 0;
  HDOG_CUDA_TRY(cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  if (status) return fail(status, "hdog_dog: a bounded device wait hit its limit");
  return HDOG_OK;
}

extern "C" int hdog_hessian_pd(hdog_ctx *c, const float *d_dog, uint8_t *d_mask, float *d_hessian, void *stream) {
  CTX_GUARD(c);
  if (!d_dog || !d_mask) return fail(HDOG_ERR_ARG, "hdog_hessian_pd: null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  TRY(single_sub(c, nullptr, st));
  launch_hessian_pd(c->d_subs, 1, c->W, c->H, c->D, d_dog, d_mask, d_hessian, st);
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

extern "C" int hdog_ccl(hdog_ctx *c, const uint8_t *d_mask, int32_t *d_labels, void *stream) {
  CTX_GUARD(c);
  if (!d_mask || !d_labels) return fail(HDOG_ERR_ARG, "hdog_ccl: null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  TRY(single_sub(c, nullptr, st));
  zero_async(c->status, sizeof(int), st);
  launch_ccl(c->d_subs, 1, c->W, c->H, c->D, c->nvox, d_mask, d_labels, c->edges, c->edge_count, c->root_bits,
             c->blk_counts, c->status, c->num_sms, st);
  HDOG_CUDA_TRY(cudaGetLastError());
  int status = 0;
  HDOG_CUDA_TRY(cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  if (status) return fail(status, "device loop limit reached in connected-component labelling");
  return HDOG_OK;
}

extern "C" int hdog_regional_features(hdog_ctx *c, const int32_t *d_labels, const float *d_norm,
                                      const float *d_dog, hdog_regions *out, void *stream) {
  CTX_GUARD(c);
  if (!d_labels || !d_norm || !d_dog || !out) return fail(HDOG_ERR_ARG, "hdog_regional_features: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  TRY(single_sub(c, nullptr, st));
  zero_async(c->status, sizeof(int), st);
  // foreground = nonzero label; roots = voxels labelled with their own index
  launch_roots_from_labels(c->d_subs, 1, c->nvox, d_labels, c->mask, c->root_bits, c->blk_counts, st);
  int32_t *rank = reinterpret_cast<int32_t *>(c->fa);
  launch_regions(c->d_subs, 1, c->nvox, vseg_of(c), c->mask, d_labels, c->root_bits, d_norm, d_dog, rank,
                 c->blk_counts, c->blk_offsets, c->chunk, c->num_regions, c->acc, c->slots, c->status, st);
  launch_finalize(c->d_subs, 1, c->reg_cap, rseg_of(c), c->num_regions, c->acc, c->slots, c->out,
                  filter_of(c->p, true), c->blk_counts, c->blk_offsets, c->chunk, c->num_records, c->records, c->nblk, st);
  HDOG_CUDA_TRY(cudaGetLastError());
  int64_t nr = 0;
  int status = 0;
  HDOG_CUDA_TRY(cudaMemcpyAsync(&nr, c->num_regions, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  HDOG_CUDA_TRY(cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, st));
  HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  if (status == HDOG_ERR_CAPACITY) return fail(HDOG_ERR_CAPACITY, "region capacity exceeded");
  if (status) return fail(status, "regional features failed");
  out->num_regions = nr;
  out->label = c->acc.label;
  out->count = c->acc.count;
  out->intensity = c->out.intensity;
  out->centroid = c->out.centroid;
  out->hessian = c->out.hessian;
  out->eigen = c->out.eigen;
  out->pitch = c->slots;
  return HDOG_OK;
}

extern "C" int hdog_erosion(hdog_ctx *c, const uint16_t *d_src, uint16_t *d_dst, int rxy, int rz, void *stream) {
  CTX_GUARD(c);
  if (!d_src || !d_dst) return fail(HDOG_ERR_ARG, "hdog_erosion: null buffer");
  if (rxy < 0 || rz < 0 || rxy > kMaxRadiusXY || rz > 1000)
    return fail(HDOG_ERR_SHAPE, "hdog_erosion: radius out of range");
  cudaStream_t st = (cudaStream_t)stream;
  TRY(single_sub(c, d_src, st));
  // the erosion writes dst at S.vox = 0; its scratch is fa (two packed volumes)
  launch_erosion(c->d_subs, 1, c->W, c->H, c->D, rxy, rz, srcs_aligned8(c, 1), reinterpret_cast<uint32_t *>(c->fa),
                 d_dst, st);
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

// ------------------------------------------------------------------ whole chain
extern "C" int hdog_run_substack(hdog_ctx *c, const uint16_t *img, int img_on_device, int depth_valid, int z0,
                                 hdog_record *out, int64_t cap, int64_t *n_records, void *stream) {
  CTX_GUARD(c);
  if (!img || !n_records || (cap > 0 && !out)) return fail(HDOG_ERR_ARG, "hdog_run_substack: null argument");
  if (depth_valid < 1 || depth_valid > c->D) return fail(HDOG_ERR_ARG, "depth_valid must be in [1, depth]");
  cudaStream_t st = (cudaStream_t)stream;
  const uint16_t *src = img;
  if (!img_on_device) {
    HDOG_CUDA_TRY(cudaMemcpyAsync(c->img, img, (size_t)depth_valid * c->W * c->H * sizeof(uint16_t),
                                  cudaMemcpyHostToDevice, st));
    src = c->img;
  }
  set_sub(c, 0, src, depth_valid, z0);
  c->last.clear();
  TRY(run_batch(c, 1, st));
  TRY(collect_records(c, 1, c->last, st));
  return copy_out(c->last, out, cap, n_records);
}

// z0 schedule of HDoG3D_main.cpp:309-314.
static int schedule(int length, int D, int m, std::vector<int> &z0s) {
  z0s.clear();
  if (length - m <= 0) return HDOG_OK;
  const int stride = D - 2 * m;
  if (stride <= 0) return fail(HDOG_ERR_PARAM, "depth must exceed twice the depth margin");
  for (int z0 = 0; z0 < length - m; z0 += stride) z0s.push_back(z0);
  return HDOG_OK;
}

static int run_stack_locked(hdog_ctx *c, const uint16_t *stack, int on_device, int length, RecordBuf &out,
                            cudaStream_t st, hdog_record *direct = nullptr, int64_t direct_cap = 0) {
  std::vector<int> z0s;
  TRY(schedule(length, c->D, c->margin, z0s));
  if (z0s.empty()) return HDOG_OK;
  const size_t plane = (size_t)c->W * c->H;
  const uint16_t *dev = stack;
  // batches of as many substacks as the context holds.  With host input the first batch
  // holds host_batch substacks, so that only its slices are copied before work starts, and
  // each later batch at most twice the one before: its slices are copied while the one
  // before runs, and a batch's compute takes several times longer than the copy of twice
  // its new slices (a 32-slice substack adds 16 new slices), so no batch waits for its chunk.
  std::vector<size_t> starts;   // first substack of each batch, then the end
  {
    const size_t full = (size_t)c->max_sub, n = z0s.size();
    size_t size = full;
    if (!on_device && c->host_batch > 0) size = std::min(full, (size_t)c->host_batch);
    for (size_t b0 = 0; b0 < n;) {
      starts.push_back(b0);
      size_t take = std::min(size, n - b0);
      const size_t next = std::min(full, 2 * size);
      // a remainder smaller than half the next batch joins this one when the context holds it
      if (!on_device && n - b0 - take > 0 && n - b0 - take < (next + 1) / 2 && n - b0 <= full) take = n - b0;
      b0 += take;
      size = on_device ? full : next;
    }
    starts.push_back(n);
  }
  const size_t nbatch = starts.size() - 1;
  // With host input and a first batch of one substack, a short last substack (one whose
  // slices end before its depth, the rest being the zero tail) runs first: it needs only its
  // own slices, so the GPU starts after fewer of them are copied (16 instead of 32 for a
  // 128-slice stack in substacks of 32).  Its records are held aside and appended after the
  // others, so they come out in the schedule's order.
  const size_t n_sub_all = z0s.size();
  const bool last_first = !on_device && nbatch >= 2 && starts[1] == 1 &&
                          length - z0s.back() < std::min(c->D, length - z0s.front());
  std::vector<int> order(n_sub_all);
  for (size_t k = 0; k < n_sub_all; k++) order[k] = z0s[last_first ? (k + n_sub_all - 1) % n_sub_all : k];
  // on an early error return the chunk copies may still be reading the caller's host
  // stack: wait for them, so the caller can free or reuse it once the call returns
  struct CopyWait {
    cudaStream_t st = nullptr;
    bool armed = false;
    ~CopyWait() {
      if (armed) cudaStreamSynchronize(st);
    }
  } copy_wait;
  if (!on_device) {
    const size_t bytes = (size_t)length * plane * sizeof(uint16_t);
    if (bytes > c->stack_bytes) {
      if (c->stack_buf) cudaFree(c->stack_buf);
      c->stack_buf = nullptr;
      c->stack_bytes = 0;
      if (cudaMalloc(&c->stack_buf, bytes) != cudaSuccess)
        return fail(HDOG_ERR_NOMEM, "hdog_run_stack: no device memory for the stack");
      c->stack_bytes = bytes;
    }
    if (!c->copy_st) {
      HDOG_CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_st, cudaStreamNonBlocking));
      HDOG_CUDA_TRY(cudaEventCreateWithFlags(&c->start_ev, cudaEventDisableTiming));
    }
    while (c->chunk_ev.size() < nbatch) {
      cudaEvent_t e;
      HDOG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      c->chunk_ev.push_back(e);
    }
    // the copies start after the work already queued on st (which may still read stack_buf)
    HDOG_CUDA_TRY(cudaEventRecord(c->start_ev, st));
    HDOG_CUDA_TRY(cudaStreamWaitEvent(c->copy_st, c->start_ev, 0));
    copy_wait.st = c->copy_st;
    copy_wait.armed = true;
    // slices [0, z_done) and [tail_from, length) are on their way
    size_t z_done = 0, tail_from = (size_t)length;
    for (size_t b = 0; b < nbatch; b++) {
      if (b == 0 && last_first) {
        tail_from = (size_t)z0s.back();
        HDOG_CUDA_TRY(cudaMemcpyAsync(c->stack_buf + tail_from * plane, stack + tail_from * plane,
                                      ((size_t)length - tail_from) * plane * sizeof(uint16_t),
                                      cudaMemcpyHostToDevice, c->copy_st));
      } else {
        const size_t last = starts[b + 1] - 1;
        const size_t z_end = std::min(tail_from, (size_t)order[last] + (size_t)c->D);
        if (z_end > z_done) {
          HDOG_CUDA_TRY(cudaMemcpyAsync(c->stack_buf + z_done * plane, stack + z_done * plane,
                                        (z_end - z_done) * plane * sizeof(uint16_t), cudaMemcpyHostToDevice,
                                        c->copy_st));
          z_done = z_end;
        }
      }
      HDOG_CUDA_TRY(cudaEventRecord(c->chunk_ev[b], c->copy_st));
    }
    dev = c->stack_buf;
  }
  for (size_t b = 0; b < nbatch; b++) {
    const size_t first = starts[b];
    const int nsub = (int)(starts[b + 1] - first);
    if (!on_device && c->timer) {
      // time the GPU would wait for this batch's chunk: sync on it while timing
      HostPhase ph(c, "host_wait_chunk");
      HDOG_CUDA_TRY(cudaEventSynchronize(c->chunk_ev[b]));
    }
    if (!on_device) HDOG_CUDA_TRY(cudaStreamWaitEvent(st, c->chunk_ev[b], 0));
    for (int s = 0; s < nsub; s++) {
      const int z0 = order[first + s];
      set_sub(c, s, dev + (size_t)z0 * plane, std::min(c->D, length - z0), z0);
    }
    TRY(run_batch(c, nsub, st));
    if (b == 0 && last_first) {
      c->aside.clear();
      TRY(collect_records(c, nsub, c->aside, st));
    } else {
      TRY(collect_records(c, nsub, out, st, direct, direct_cap));
    }
  }
  copy_wait.armed = false;   // every batch waited for its chunk, so the copies are done
  if (last_first && c->aside.n > 0) {
    if (!out.reserve(out.n + c->aside.n)) return fail(HDOG_ERR_NOMEM, "page-locked host buffer for the records failed");
    memcpy(out.p + out.n, c->aside.p, c->aside.n * sizeof(hdog_record));
    if (direct && (int64_t)(out.n + c->aside.n) <= direct_cap)
      memcpy(direct + out.n, c->aside.p, c->aside.n * sizeof(hdog_record));
    out.n += c->aside.n;
  }
  return HDOG_OK;
}

extern "C" int hdog_run_stack(hdog_ctx *c, const uint16_t *stack, int stack_on_device, int length,
                              hdog_record *out, int64_t cap, int64_t *n_records, void *stream) {
  CTX_GUARD(c);
  if (!stack || !n_records || length < 0 || (cap > 0 && !out)) return fail(HDOG_ERR_ARG, "hdog_run_stack: bad argument");
  c->last.clear();
  // a page-locked output buffer receives the records straight from the device, batch by
  // batch, so the copy out of the library's own buffer is skipped when they all fit
  hdog_record *direct = nullptr;
  if (cap > 0) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, out) == cudaSuccess && a.type == cudaMemoryTypeHost) direct = out;
    cudaGetLastError();   // a pointer unknown to CUDA is not an error here
  }
  TRY(run_stack_locked(c, stack, stack_on_device, length, c->last, (cudaStream_t)stream, direct, cap));
  if (direct && (int64_t)c->last.n <= cap) {
    *n_records = (int64_t)c->last.n;
    return HDOG_OK;
  }
  HostPhase ph(c, "host_copy_out");
  return copy_out(c->last, out, cap, n_records);
}

extern "C" int hdog_run_stacks(hdog_ctx *c, const hdog_stack_in *stacks, int n_stacks, hdog_record *out,
                               int64_t cap, int64_t *n_records, int64_t *stack_counts, void *stream) {
  CTX_GUARD(c);
  if (!n_records || n_stacks < 0 || (n_stacks > 0 && !stacks) || (cap > 0 && !out))
    return fail(HDOG_ERR_ARG, "hdog_run_stacks: bad argument");
  for (int i = 0; i < n_stacks; i++)
    if ((!stacks[i].data && stacks[i].length > 0) || stacks[i].length < 0)
      return fail(HDOG_ERR_ARG, "hdog_run_stacks: bad stack");
  cudaStream_t st = (cudaStream_t)stream;
  c->last.clear();
  if (stack_counts)
    for (int i = 0; i < n_stacks; i++) stack_counts[i] = 0;
  const size_t plane = (size_t)c->W * c->H;
  // every stack's substacks, stack by stack
  struct Item { int stack, z0; };
  std::vector<Item> items;
  std::vector<int> z0s;
  for (int i = 0; i < n_stacks; i++) {
    TRY(schedule(stacks[i].length, c->D, c->margin, z0s));
    for (int z0 : z0s) items.push_back({i, z0});
  }
  // host stacks go to device buffers of this call
  std::vector<uint16_t *> dev(n_stacks, nullptr), owned;
  struct Free {
    std::vector<uint16_t *> &v;
    ~Free() { for (uint16_t *p : v) cudaFree(p); }
  } free_owned{owned};
  for (int i = 0; i < n_stacks; i++) {
    if (stacks[i].on_device) {
      dev[i] = const_cast<uint16_t *>(stacks[i].data);
      continue;
    }
    const size_t bytes = (size_t)stacks[i].length * plane * sizeof(uint16_t);
    if (!bytes) continue;
    uint16_t *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) return fail(HDOG_ERR_NOMEM, "hdog_run_stacks: no device memory for a stack");
    owned.push_back(d);
    HDOG_CUDA_TRY(cudaMemcpyAsync(d, stacks[i].data, bytes, cudaMemcpyHostToDevice, st));
    dev[i] = d;
  }
  for (size_t b = 0; b < items.size(); b += (size_t)c->max_sub) {
    const int nsub = (int)std::min(items.size() - b, (size_t)c->max_sub);
    for (int s = 0; s < nsub; s++) {
      const Item &it = items[b + s];
      set_sub(c, s, dev[it.stack] + (size_t)it.z0 * plane, std::min(c->D, stacks[it.stack].length - it.z0), it.z0);
    }
    TRY(run_batch(c, nsub, st));
    if (stack_counts)
      for (int s = 0; s < nsub; s++) stack_counts[items[b + s].stack] += c->h_counts[s];
    TRY(collect_records(c, nsub, c->last, st));
  }
  return copy_out(c->last, out, cap, n_records);
}

// ------------------------------------------------------------------ autotuner
// Launch shapes of the two sweeps (one block per tile, or a persistent grid of a few
// blocks per SM over the device work queue) and the substacks per launch of the graph
// form, chosen by timing the caller's own first batch with CUDA events.  Results are cached
// per device, frame shape, depth, tap radii, normalization radii and context size: every
// candidate gives the same output, only the time differs.
struct TuneResult {
  LaunchShape shape;
  int batch = 0;
  std::string report;   // JSON of the timings behind the choice
};
static std::mutex g_tune_mu;
static std::vector<std::pair<std::string, TuneResult>> g_tune_cache;

static std::string tune_key(const hdog_ctx *c) {
  char k[256];
  snprintf(k, sizeof(k), "%d:%dx%dx%d:%d,%d,%d,%d:%d,%d:%d:%d", c->dev, c->W, c->H, c->D, c->taps.r[0], c->taps.r[1],
           c->taps.r[2], c->taps.r[3], c->p.radius_norm_xy, c->p.radius_norm_z, c->max_sub,
           (c->p.erosion_radius_xy || c->p.erosion_radius_z) ? 1 : 0);
  return k;
}

static bool tune_lookup(hdog_ctx *c) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  const std::string k = tune_key(c);
  for (auto &e : g_tune_cache)
    if (e.first == k) {
      c->shape = e.second.shape;
      c->shape.num_sms = c->num_sms;
      c->graph_batch = e.second.batch;
      c->tune_report = e.second.report;
      c->tuned = true;
      return true;
    }
  return false;
}

// Milliseconds of each kernel name in the timer since the last collect.
static double timer_ms(EventTimer &t, const char *name) {
  for (auto &e : t.totals)
    if (e.first == name) return e.second.ms;
  return 0.0;
}

// Tunes the context on the batch of nsub substacks whose host descriptors are set (their
// inputs in device memory).  Leaves the context's scratch with one of the runs' results.
static int tune_batch(hdog_ctx *c, int nsub, cudaStream_t st) {
  if (c->tuned || tune_lookup(c)) return HDOG_OK;
  KernelTimer *saved = g_timer;
  EventTimer timer;
  g_timer = &timer;
  struct Restore {
    KernelTimer *saved;
    ~Restore() { g_timer = saved; }
  } restore{saved};
  const bool fused = fused_ok(c);
  struct Cand {
    int dog, hess;
  };
  // grid form, and persistent grids at and below the sweeps' occupancy (three DoG blocks,
  // five Hessian blocks per SM)
  const Cand cands[] = {{0, 0}, {3, 5}, {2, 4}};
  double dog_ms[3] = {0, 0, 0}, hess_ms[3] = {0, 0, 0}, all_ms[3] = {0, 0, 0};
  c->shape = LaunchShape{};
  c->shape.num_sms = c->num_sms;
  TRY(enqueue_batch(c, nsub, fused, st));   // warm-up
  HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  timer.collect();
  timer.totals.clear();
  for (int i = 0; i < (fused ? 3 : 1); i++) {
    c->shape.dog_per_sm = cands[i].dog;
    c->shape.hess_per_sm = cands[i].hess;
    TRY(enqueue_batch(c, nsub, fused, st));
    HDOG_CUDA_TRY(cudaStreamSynchronize(st));
    timer.collect();
    dog_ms[i] = timer_ms(timer, "k_dog_sweep");
    hess_ms[i] = timer_ms(timer, "k_hess_sweep");
    for (auto &e : timer.totals) all_ms[i] += e.second.ms;
    timer.totals.clear();
  }
  int bd = 0, bh = 0;
  for (int i = 1; i < (fused ? 3 : 1); i++) {
    if (dog_ms[i] < dog_ms[bd]) bd = i;
    if (hess_ms[i] < hess_ms[bh]) bh = i;
  }
  c->shape.dog_per_sm = cands[bd].dog;
  c->shape.hess_per_sm = cands[bh].hess;
  // substacks per launch: the full batch against half of it, by time per substack of the chain
  int batch = nsub;
  double half_ms = 0.0, full_ms = 0.0;
  {
    TRY(enqueue_batch(c, nsub, fused, st));
    HDOG_CUDA_TRY(cudaStreamSynchronize(st));
    timer.collect();
    for (auto &e : timer.totals) full_ms += e.second.ms;
    timer.totals.clear();
    if (nsub >= 2) {
      const int h = nsub / 2;
      TRY(enqueue_batch(c, h, fused, st));
      HDOG_CUDA_TRY(cudaStreamSynchronize(st));
      timer.collect();
      for (auto &e : timer.totals) half_ms += e.second.ms;
      timer.totals.clear();
      if (half_ms / h < full_ms / nsub) batch = h;
    }
  }
  c->graph_batch = batch;
  char rep[768];
  snprintf(rep, sizeof(rep),
           "{\"frame\": [%d, %d, %d], \"tuned_on_substacks\": %d, \"candidates\": [[0, 0], [3, 5], [2, 4]], "
           "\"k_dog_sweep_ms\": [%.4f, %.4f, %.4f], \"k_hess_sweep_ms\": [%.4f, %.4f, %.4f], "
           "\"dog_per_sm\": %d, \"hess_per_sm\": %d, \"chain_ms_full_batch\": %.4f, \"chain_ms_half_batch\": %.4f, "
           "\"batch\": %d}",
           c->W, c->H, c->D, nsub, dog_ms[0], dog_ms[1], dog_ms[2], hess_ms[0], hess_ms[1], hess_ms[2],
           c->shape.dog_per_sm, c->shape.hess_per_sm, full_ms, half_ms, batch);
  c->tune_report = rep;
  c->tuned = true;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache.emplace_back(tune_key(c), TuneResult{c->shape, batch, c->tune_report});
  return HDOG_OK;
}

extern "C" int hdog_autotune(hdog_ctx *c, const uint16_t *d_stack, int length, void *stream) {
  CTX_GUARD(c);
  if (!d_stack || length < 1) return fail(HDOG_ERR_ARG, "hdog_autotune: bad argument");
  std::vector<int> z0s;
  TRY(schedule(length, c->D, c->margin, z0s));
  if (z0s.empty()) return fail(HDOG_ERR_ARG, "hdog_autotune: the stack has no substack");
  const int nsub = (int)std::min(z0s.size(), (size_t)c->max_sub);
  const size_t plane = (size_t)c->W * c->H;
  for (int s = 0; s < nsub; s++)
    set_sub(c, s, d_stack + (size_t)z0s[s] * plane, std::min(c->D, length - z0s[s]), z0s[s]);
  c->tuned = false;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const std::string k = tune_key(c);
    for (size_t i = 0; i < g_tune_cache.size(); i++)
      if (g_tune_cache[i].first == k) {
        g_tune_cache.erase(g_tune_cache.begin() + i);
        break;
      }
  }
  return tune_batch(c, nsub, (cudaStream_t)stream);
}

extern "C" int hdog_ctx_tuning(hdog_ctx *c, char *buf, size_t cap) {
  if (!c || !buf || cap == 0) return fail(HDOG_ERR_ARG, "hdog_ctx_tuning: bad argument");
  std::lock_guard<std::mutex> lock(c->mu);
  const std::string &r = c->tuned ? c->tune_report : std::string("{}");
  if (r.size() + 1 > cap) return fail(HDOG_ERR_CAPACITY, "hdog_ctx_tuning: buffer too small");
  memcpy(buf, r.c_str(), r.size() + 1);
  return HDOG_OK;
}

// ------------------------------------------------------------------ the batched graph form
struct hdog_graph {
  int dev = 0;
  std::vector<hdog_ctx *> ctxs;          // distinct contexts, in locking order
  std::vector<hdog_graph_stack> stacks;
  std::vector<hdog_ctx *> stack_ctx;     // the context of each stack
  std::vector<int64_t> stack_first;      // run index of each stack's first substack
  std::vector<int64_t> stack_nsub;
  int64_t n_sub = 0;
  int64_t out_cap = 0;
  void *dmem = nullptr;                  // header (total, redo) | slot table | records
  int64_t *d_total = nullptr;
  int *d_redo = nullptr;
  GraphSlot *d_table = nullptr;
  hdog_record *d_out = nullptr;
  int64_t *h_hdr = nullptr;              // pinned: total, redo, then the slot table
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  RecordBuf staged;                      // the run's records as placed on the device
  RecordBuf last;                        // the last run's records in the caller's order
  std::vector<int64_t> last_counts;
  std::mutex mu;
};

// Locks the contexts of a graph in a fixed order for the duration of a call.
struct CtxLocks {
  std::vector<std::unique_lock<std::mutex>> held;
  explicit CtxLocks(const std::vector<hdog_ctx *> &cs) {
    for (hdog_ctx *c : cs) held.emplace_back(c->mu);
  }
};

extern "C" int hdog_graph_destroy(hdog_graph *g) {
  if (!g) return HDOG_OK;
  cudaSetDevice(g->dev);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->dmem) cudaFree(g->dmem);
  if (g->h_hdr) cudaFreeHost(g->h_hdr);
  g->staged.release();
  g->last.release();
  delete g;
  return HDOG_OK;
}

extern "C" int hdog_graph_create(hdog_ctx *const *ctxs, int n_ctx, const hdog_graph_stack *stacks, int n_stacks,
                                 void *stream, hdog_graph **out) {
  if (!out) return fail(HDOG_ERR_ARG, "hdog_graph_create: null output pointer");
  *out = nullptr;
  if (!ctxs || n_ctx < 1 || n_stacks < 0 || (n_stacks > 0 && !stacks))
    return fail(HDOG_ERR_ARG, "hdog_graph_create: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  std::unique_ptr<hdog_graph, int (*)(hdog_graph *)> g(new hdog_graph(), hdog_graph_destroy);
  for (int i = 0; i < n_ctx; i++) {
    if (!ctxs[i]) return fail(HDOG_ERR_ARG, "hdog_graph_create: null context");
    if (ctxs[i]->dev != ctxs[0]->dev) return fail(HDOG_ERR_ARG, "hdog_graph_create: contexts on different devices");
    if (ctxs[i]->max_sub > kGraphMaxBatch)
      return fail(HDOG_ERR_ARG, "hdog_graph_create: contexts of at most " + std::to_string(kGraphMaxBatch) + " substacks");
    for (int j = 0; j < i; j++)
      if (ctxs[j] == ctxs[i] || (ctxs[j]->W == ctxs[i]->W && ctxs[j]->H == ctxs[i]->H))
        return fail(HDOG_ERR_ARG, "hdog_graph_create: one context per frame shape");
    g->ctxs.push_back(ctxs[i]);
  }
  std::sort(g->ctxs.begin(), g->ctxs.end());
  g->dev = ctxs[0]->dev;
  HDOG_CUDA_TRY(cudaSetDevice(g->dev));
  CtxLocks locks(g->ctxs);
  // every stack's substacks in the caller's order; each stack goes to the context of its frame
  std::vector<std::vector<int>> z0_of(n_stacks);
  int64_t processed = 0;
  for (int i = 0; i < n_stacks; i++) {
    const hdog_graph_stack &sp = stacks[i];
    if (!sp.data || sp.length < 0) return fail(HDOG_ERR_ARG, "hdog_graph_create: bad stack");
    hdog_ctx *c = nullptr;
    for (hdog_ctx *x : g->ctxs)
      if (x->W == sp.width && x->H == sp.height) c = x;
    if (!c) return fail(HDOG_ERR_ARG, "hdog_graph_create: no context for a stack's frame shape");
    TRY(schedule(sp.length, c->D, c->margin, z0_of[i]));
    g->stacks.push_back(sp);
    g->stack_ctx.push_back(c);
    g->stack_first.push_back(g->n_sub);
    g->stack_nsub.push_back((int64_t)z0_of[i].size());
    g->n_sub += (int64_t)z0_of[i].size();
    processed += (int64_t)z0_of[i].size() * c->nvox;
  }
  g->out_cap = std::max<int64_t>(65536, processed / 512);
  const size_t table_bytes = align256((size_t)std::max<int64_t>(g->n_sub, 1) * sizeof(GraphSlot));
  if (cudaMalloc(&g->dmem, 256 + table_bytes + (size_t)g->out_cap * sizeof(hdog_record)) != cudaSuccess)
    return fail(HDOG_ERR_NOMEM, "hdog_graph_create: no device memory for the run's records");
  g->d_total = (int64_t *)g->dmem;
  g->d_redo = (int *)((char *)g->dmem + 8);
  g->d_table = (GraphSlot *)((char *)g->dmem + 256);
  g->d_out = (hdog_record *)((char *)g->dmem + 256 + table_bytes);
  if (cudaMallocHost(&g->h_hdr, 16 + (size_t)std::max<int64_t>(g->n_sub, 1) * sizeof(GraphSlot)) != cudaSuccess)
    return fail(HDOG_ERR_NOMEM, "hdog_graph_create: pinned host memory");
  // per context: its substacks (stack by stack), the first batch tunes the launch shapes
  struct Item {
    int stack;
    int z0;
    int64_t id;
  };
  std::vector<std::vector<Item>> items(g->ctxs.size());
  for (int i = 0; i < n_stacks; i++) {
    const size_t k = std::find(g->ctxs.begin(), g->ctxs.end(), g->stack_ctx[i]) - g->ctxs.begin();
    for (size_t j = 0; j < z0_of[i].size(); j++) items[k].push_back({i, z0_of[i][j], g->stack_first[i] + (int64_t)j});
  }
  auto set_item = [&](hdog_ctx *c, int s, const Item &it) {
    const hdog_graph_stack &sp = g->stacks[it.stack];
    set_sub(c, s, sp.data + (size_t)it.z0 * c->W * c->H, std::min(c->D, sp.length - it.z0), it.z0);
  };
  for (size_t k = 0; k < g->ctxs.size(); k++) {
    hdog_ctx *c = g->ctxs[k];
    if (items[k].empty()) continue;
    const int nsub = (int)std::min(items[k].size(), (size_t)c->max_sub);
    for (int s = 0; s < nsub; s++) set_item(c, s, items[k][s]);
    TRY(tune_batch(c, nsub, st));
  }
  // capture every batch of every context, with the record placement after each, on a
  // stream of its own (the caller's may be the legacy default stream, which cannot capture)
  HDOG_CUDA_TRY(cudaStreamSynchronize(st));
  struct CapStream {
    cudaStream_t s = nullptr;
    ~CapStream() {
      if (s) cudaStreamDestroy(s);
    }
  } cap;
  HDOG_CUDA_TRY(cudaStreamCreateWithFlags(&cap.s, cudaStreamNonBlocking));
  st = cap.s;
  KernelTimer *saved_timer = g_timer;
  g_timer = nullptr;
  HDOG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int rc = HDOG_OK;
  zero_async(g->dmem, 256, st);
  for (size_t k = 0; k < g->ctxs.size() && rc == HDOG_OK; k++) {
    hdog_ctx *c = g->ctxs[k];
    const bool fused = fused_ok(c);
    const size_t per = (size_t)std::max(1, c->graph_batch > 0 ? c->graph_batch : c->max_sub);
    for (size_t b = 0; b < items[k].size() && rc == HDOG_OK; b += per) {
      const int nsub = (int)std::min(per, items[k].size() - b);
      GraphIds ids{};
      for (int s = 0; s < nsub; s++) {
        set_item(c, s, items[k][b + s]);
        ids.id[s] = (int)items[k][b + s].id;
      }
      rc = enqueue_batch(c, nsub, fused, st);
      if (rc != HDOG_OK) break;
      launch_graph_place(nsub, ids, c->num_records, c->fg_count, c->fg_cap, fused, c->status, g->d_total, g->d_table,
                         g->d_redo, g->out_cap, st);
      launch_graph_copy(nsub, ids, c->records, c->reg_cap, g->d_table, g->d_out, g->out_cap, st);
    }
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(st, &graph);
  g_timer = saved_timer;
  if (rc != HDOG_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ec != cudaSuccess) return hdog_set_cuda_error(ec, "hdog_graph_create: stream capture");
  g->graph = graph;
  HDOG_CUDA_TRY(cudaGraphInstantiate(&g->exec, g->graph, 0));
  *out = g.release();
  return HDOG_OK;
}

extern "C" int hdog_graph_run(hdog_graph *g, hdog_record *out, int64_t cap, int64_t *n_records, int64_t *stack_counts,
                              void *stream) {
  if (!g || !n_records || (cap > 0 && !out)) return fail(HDOG_ERR_ARG, "hdog_graph_run: bad argument");
  std::lock_guard<std::mutex> glock(g->mu);
  HDOG_CUDA_TRY(cudaSetDevice(g->dev));
  cudaStream_t st = (cudaStream_t)stream;
  const size_t nst = g->stacks.size();
  g->last.clear();
  g->last_counts.assign(nst, 0);
  bool redo = false;
  {
    CtxLocks locks(g->ctxs);
    HDOG_CUDA_TRY(cudaGraphLaunch(g->exec, st));
    HDOG_CUDA_TRY(cudaMemcpyAsync(g->h_hdr, g->dmem, 16, cudaMemcpyDeviceToHost, st));
    if (g->n_sub > 0)
      HDOG_CUDA_TRY(cudaMemcpyAsync(g->h_hdr + 2, g->d_table, (size_t)g->n_sub * sizeof(GraphSlot),
                                    cudaMemcpyDeviceToHost, st));
    HDOG_CUDA_TRY(cudaStreamSynchronize(st));
    const int64_t total = g->h_hdr[0];
    redo = (int)(g->h_hdr[1] & 0xFFFFFFFF) != 0 || total > g->out_cap;
    if (!redo) {
      if (!g->staged.reserve((size_t)total) || !g->last.reserve((size_t)total))
        return fail(HDOG_ERR_NOMEM, "page-locked host buffer for the records failed");
      if (total > 0)
        HDOG_CUDA_TRY(cudaMemcpyAsync(g->staged.p, g->d_out, (size_t)total * sizeof(hdog_record), cudaMemcpyDeviceToHost,
                                      st));
      HDOG_CUDA_TRY(cudaStreamSynchronize(st));
      g->staged.n = (size_t)total;
      const GraphSlot *table = reinterpret_cast<const GraphSlot *>(g->h_hdr + 2);
      // the substacks' records in the caller's order: stack by stack, substack by substack
      std::vector<std::pair<size_t, size_t>> pieces;
      pieces.reserve((size_t)g->n_sub);
      size_t n = 0;
      for (size_t i = 0; i < nst; i++)
        for (int64_t j = 0; j < g->stack_nsub[i]; j++) {
          const GraphSlot &sl = table[g->stack_first[i] + j];
          if (sl.count > 0) pieces.emplace_back((size_t)sl.off, (size_t)sl.count);
          n += (size_t)sl.count;
          g->last_counts[i] += sl.count;
        }
      host_gather(g->last.p, g->staged.p, pieces, n);
      g->last.n = n;
    }
  }
  if (redo) {
    // a batch needed the host's fallback (foreground list or region capacity, a bounded
    // loop, or more records than the run's array holds): rerun stack by stack without the graph
    g->last.clear();
    for (size_t i = 0; i < nst; i++) {
      hdog_ctx *c = g->stack_ctx[i];
      std::lock_guard<std::mutex> lock(c->mu);
      const size_t before = g->last.n;
      TRY(run_stack_locked(c, g->stacks[i].data, 1, g->stacks[i].length, g->last, st));
      g->last_counts[i] = (int64_t)(g->last.n - before);
    }
  }
  if (stack_counts)
    for (size_t i = 0; i < nst; i++) stack_counts[i] = g->last_counts[i];
  return copy_out(g->last, out, cap, n_records);
}

extern "C" int hdog_graph_last_records(hdog_graph *g, hdog_record *out, int64_t cap, int64_t *n_records) {
  if (!g || !n_records || (cap > 0 && !out)) return fail(HDOG_ERR_ARG, "hdog_graph_last_records: bad argument");
  std::lock_guard<std::mutex> lock(g->mu);
  return copy_out(g->last, out, cap, n_records);
}

// ------------------------------------------------------------------ differentiable chain
extern "C" size_t hdog_soft_workspace_bytes(const hdog_soft_params *p) { return p ? soft_workspace_bytes(*p) : 0; }

extern "C" int hdog_soft_forward(const hdog_soft_params *p, const float *d_volume, const int32_t *d_pos, int n_pos,
                                 const int32_t *d_neg, int n_neg, float *d_loss, float *d_scores, void *d_workspace,
                                 void *stream) {
  const int rc = soft_forward(p, d_volume, d_pos, n_pos, d_neg, n_neg, d_loss, d_scores, d_workspace,
                              (cudaStream_t)stream);
  if (rc != HDOG_OK) return fail(rc, "hdog_soft_forward: bad argument, parameter or sigma");
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

extern "C" int hdog_soft_backward(const hdog_soft_params *p, const float *d_volume, const int32_t *d_pos, int n_pos,
                                  const int32_t *d_neg, int n_neg, float grad_loss, float *d_grad_volume,
                                  float *d_grad_sigma, float *d_grad_thresh, void *d_workspace, void *stream) {
  const int rc = soft_backward(p, d_volume, d_pos, n_pos, d_neg, n_neg, grad_loss, d_grad_volume, d_grad_sigma,
                               d_grad_thresh, d_workspace, (cudaStream_t)stream);
  if (rc != HDOG_OK) return fail(rc, "hdog_soft_backward: bad argument, parameter or sigma");
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

extern "C" int hdog_soft_backward_kept(const hdog_soft_params *p, const float *d_volume, const int32_t *d_pos,
                                       int n_pos, const int32_t *d_neg, int n_neg, float grad_loss,
                                       float *d_grad_volume, float *d_grad_sigma, float *d_grad_thresh,
                                       void *d_workspace, void *stream) {
  const int rc = soft_backward(p, d_volume, d_pos, n_pos, d_neg, n_neg, grad_loss, d_grad_volume, d_grad_sigma,
                               d_grad_thresh, d_workspace, (cudaStream_t)stream, true);
  if (rc != HDOG_OK) return fail(rc, "hdog_soft_backward_kept: bad argument, parameter or sigma");
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

// ------------------------------------------------------------------ after the records
extern "C" int hdog_records_to_global(const hdog_record *d_records, int64_t n, const hdog_global_params *p,
                                      hdog_global *d_out, void *stream) {
  if (!p || n < 0 || (n > 0 && (!d_records || !d_out))) return fail(HDOG_ERR_ARG, "hdog_records_to_global: bad argument");
  if (p->promote != HDOG_PROMOTE_F32 && p->promote != HDOG_PROMOTE_F64)
    return fail(HDOG_ERR_ARG, "hdog_records_to_global: promote must be HDOG_PROMOTE_F32 or HDOG_PROMOTE_F64");
  launch_to_global(d_records, n, *p, d_out, (cudaStream_t)stream);
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

extern "C" int hdog_scale_merge(const hdog_global *d_in, int64_t n, const hdog_scalemerge_params *p,
                                hdog_scalemerged *d_out, void *stream) {
  if (!p || n < 0 || (n > 0 && (!d_in || !d_out))) return fail(HDOG_ERR_ARG, "hdog_scale_merge: bad argument");
  if (p->promote != HDOG_PROMOTE_F32 && p->promote != HDOG_PROMOTE_F64)
    return fail(HDOG_ERR_ARG, "hdog_scale_merge: promote must be HDOG_PROMOTE_F32 or HDOG_PROMOTE_F64");
  launch_scale_merge(d_in, n, *p, d_out, (cudaStream_t)stream);
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

extern "C" int hdog_classifier_features(const hdog_record *d_records, int64_t n, const hdog_clf_params *p, double *d_X,
                                        void *stream) {
  if (!p || n < 0 || (n > 0 && (!d_records || !d_X))) return fail(HDOG_ERR_ARG, "hdog_classifier_features: bad argument");
  launch_clf_features(d_records, n, *p, d_X, (cudaStream_t)stream);
  HDOG_CUDA_TRY(cudaGetLastError());
  return HDOG_OK;
}

extern "C" int hdog_last_records(hdog_ctx *c, hdog_record *out, int64_t cap, int64_t *n_records) {
  if (!c || !n_records || (cap > 0 && !out)) return fail(HDOG_ERR_ARG, "hdog_last_records: bad argument");
  std::lock_guard<std::mutex> lock(c->mu);
  return copy_out(c->last, out, cap, n_records);
}

// ------------------------------------------------------------------ parameter file
static int jnum(const json::Value *o, const char *key, double &v, bool required, const std::string &where) {
  const json::Value *x = o ? o->get(key) : nullptr;
  if (!x) return required ? fail(HDOG_ERR_PARAM, "parameter file: missing " + where + key) : 1;
  if (x->kind == json::Value::Number) v = x->num;
  else if (x->kind == json::Value::Bool) v = x->b ? 1 : 0;
  else return fail(HDOG_ERR_PARAM, "parameter file: " + where + key + " is not a number");
  return HDOG_OK;
}

struct StackSpec {
  std::vector<std::string> src;
  std::string dst;
};

static int load_param_file(const char *path, hdog_params *p, std::vector<StackSpec> *stacks, int *verbose,
                           int *skip_existing = nullptr) {
  if (!path || !p) return fail(HDOG_ERR_ARG, "null argument");
  std::ifstream f(path, std::ios::binary);
  if (!f.is_open()) return fail(HDOG_ERR_IO, std::string("Unable to open file ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string text = ss.str();
  json::Value root;
  std::string err;
  if (!json::Parser(text).parse(root, err)) return fail(HDOG_ERR_PARAM, std::string("parameter file: ") + err);
  if (root.kind != json::Value::Object) return fail(HDOG_ERR_PARAM, "parameter file: top level is not an object");
  memset(p, 0, sizeof(*p));
  double v;
  TRY(jnum(&root, "devID", v, true, ""));
  p->dev_id = (int)v;
  if (verbose) {
    *verbose = 0;
    if (jnum(&root, "verbose", v, false, "") == HDOG_OK) *verbose = v != 0;
  }
  const json::Value *img = root.get("input_image_info");
  if (!img) return fail(HDOG_ERR_PARAM, "parameter file: missing input_image_info");
  TRY(jnum(img, "width", v, true, "input_image_info.")); p->width = (int)v;
  TRY(jnum(img, "height", v, true, "input_image_info.")); p->height = (int)v;
  TRY(jnum(img, "left_margin", v, true, "input_image_info.")); p->left_margin = (int)v;
  TRY(jnum(img, "right_margin", v, true, "input_image_info.")); p->right_margin = (int)v;
  TRY(jnum(img, "top_margin", v, true, "input_image_info.")); p->top_margin = (int)v;
  TRY(jnum(img, "bottom_margin", v, true, "input_image_info.")); p->bottom_margin = (int)v;
  const json::Value *co = root.get("coordinate_info");
  if (!co) return fail(HDOG_ERR_PARAM, "parameter file: missing coordinate_info");
  TRY(jnum(co, "scale_x", v, true, "coordinate_info."));
  TRY(jnum(co, "scale_y", v, true, "coordinate_info."));
  TRY(jnum(co, "scale_z", v, true, "coordinate_info."));
  const json::Value *hp = root.get("HDoG_param");
  if (!hp) return fail(HDOG_ERR_PARAM, "parameter file: missing HDoG_param");
  const std::string w = "HDoG_param.";
  TRY(jnum(hp, "depth", v, true, w)); p->depth = (int)v;
  TRY(jnum(hp, "extra_depth_margin", v, true, w)); p->extra_depth_margin = (int)v;
  const json::Value *rn = hp->get("radius_norm");
  if (!rn) return fail(HDOG_ERR_PARAM, "parameter file: missing HDoG_param.radius_norm");
  TRY(jnum(rn, "xy_large", v, true, w + "radius_norm.")); p->radius_norm_xy = (int)v;
  TRY(jnum(rn, "z_large", v, true, w + "radius_norm.")); p->radius_norm_z = (int)v;
  TRY(jnum(hp, "min_intensity", v, true, w)); p->min_intensity = (int)(uint16_t)(int64_t)v;
  TRY(jnum(hp, "gamma_n", v, true, w)); p->gamma_n = (float)v;
  const json::Value *sd = hp->get("sigma_dog");
  if (!sd) return fail(HDOG_ERR_PARAM, "parameter file: missing HDoG_param.sigma_dog");
  TRY(jnum(sd, "xy_small", v, true, w + "sigma_dog.")); p->sigma_xy_small = (float)v;
  TRY(jnum(sd, "z_small", v, true, w + "sigma_dog.")); p->sigma_z_small = (float)v;
  TRY(jnum(sd, "xy_large", v, true, w + "sigma_dog.")); p->sigma_xy_large = (float)v;
  TRY(jnum(sd, "z_large", v, true, w + "sigma_dog.")); p->sigma_z_large = (float)v;
  TRY(jnum(hp, "min_size", v, true, w)); p->min_size = (int)(uint16_t)(int64_t)v;
  if (const json::Value *er = hp->get("erosion_radius")) {
    if (jnum(er, "xy", v, false, w) == HDOG_OK) p->erosion_radius_xy = (int)v;
    if (jnum(er, "z", v, false, w) == HDOG_OK) p->erosion_radius_z = (int)v;
  }
  if (jnum(&root, "is_ave_mode", v, false, "") == HDOG_OK) p->is_ave_mode = v != 0;
  if (skip_existing) {
    *skip_existing = 0;
    if (jnum(&root, "skip_existing", v, false, "") == HDOG_OK) *skip_existing = v != 0;
  }
  if (stacks) {
    stacks->clear();
    const json::Value *st = root.get("stacks");
    if (!st || st->kind != json::Value::Array) return fail(HDOG_ERR_PARAM, "parameter file: missing stacks array");
    for (const json::Value &s : st->arr) {
      StackSpec sp;
      const json::Value *src = s.get("src_paths");
      const json::Value *dst = s.get("dst_path");
      if (!src || src->kind != json::Value::Array || !dst || dst->kind != json::Value::String)
        return fail(HDOG_ERR_PARAM, "parameter file: each stack needs src_paths[] and dst_path");
      for (const json::Value &q : src->arr) {
        if (q.kind != json::Value::String) return fail(HDOG_ERR_PARAM, "parameter file: src_paths must be strings");
        sp.src.push_back(q.str);
      }
      sp.dst = dst->str;
      stacks->push_back(std::move(sp));
    }
  }
  return HDOG_OK;
}

extern "C" int hdog_params_load_json(const char *path, hdog_params *p) {
  return load_param_file(path, p, nullptr, nullptr);
}

// loadImage (utils.h:160-173): the first W*H uint16 values of the file.  A file with
// no data is an error; a short file leaves the rest of the slice zero, where the reference
// leaves whatever its reused pinned buffer held from an earlier slice.
static int load_slice(const std::string &path, uint16_t *dst, size_t n) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return fail(HDOG_ERR_IO, "Unable to open " + path);
  size_t got = fread(dst, sizeof(uint16_t), n, f);
  fclose(f);
  if (got == 0) return fail(HDOG_ERR_IO, "Unable to read " + path);
  if (got < n) memset(dst + got, 0, (n - got) * sizeof(uint16_t));
  return HDOG_OK;
}

// Slices [0, last) of one stack read into `dst` by several threads: the slice files are
// independent, and one thread's fread of 11 MB slices moves a few GB/s, well below what the
// page cache or a disk array gives several readers.  Every slice is attempted; the error
// reported is that of the first failing slice, as a reader going in order would report it.
struct SliceRead {
  int rc = HDOG_OK;
  std::string msg;
  double seconds = 0.0;
};

static SliceRead read_slices(const std::vector<std::string> &src, int last, uint16_t *dst, size_t plane) {
  SliceRead r;
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::string> err((size_t)std::max(0, last));
  std::vector<char> bad((size_t)std::max(0, last), 0);
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int z; (z = next.fetch_add(1)) < last;)
      if (load_slice(src[(size_t)z], dst + (size_t)z * plane, plane) != HDOG_OK) {
        err[(size_t)z] = g_last_error;   // this thread's message
        bad[(size_t)z] = 1;
      }
  };
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nt = std::max(1, std::min({last, hw, 16}));
  std::vector<std::thread> th;
  for (int i = 1; i < nt; i++) {
    try {
      th.emplace_back(work);
    } catch (...) {
      break;   // the threads that started and this one share the slices
    }
  }
  work();
  for (std::thread &t : th) t.join();
  for (int z = 0; z < last; z++)
    if (bad[(size_t)z]) {
      r.rc = HDOG_ERR_IO;
      r.msg = err[(size_t)z];
      break;
    }
  r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return r;
}

// One stack's records written to "<dst>.part" and renamed to dst once complete.
static SliceRead write_records(const std::string &dst, const hdog_record *rec, int64_t n) {
  SliceRead w;
  const std::string part = dst + ".part";
  FILE *f = fopen(part.c_str(), "wb");
  if (!f) {
    w.rc = HDOG_ERR_IO;
    w.msg = "Unable to open " + part;
    return w;
  }
  if (n > 0 && fwrite(rec, sizeof(hdog_record), (size_t)n, f) != (size_t)n) {
    fclose(f);
    remove(part.c_str());
    w.rc = HDOG_ERR_IO;
    w.msg = "Unable to write " + part;
    return w;
  }
  if (fclose(f) != 0 || rename(part.c_str(), dst.c_str()) != 0) {
    remove(part.c_str());
    w.rc = HDOG_ERR_IO;
    w.msg = "Unable to write " + dst;
  }
  return w;
}

// Each stack's records go to "<dst_path>.part" and are renamed to dst_path once the stack is
// complete, so an interrupted run leaves no truncated result (the reference removes dst_path
// and appends substack by substack, HDoG3D_main.cpp:295-300, utils.h:216,246; the finished
// file is the same).  With the top-level key "skip_existing" (not a reference key; default
// false) a stack whose dst_path exists is skipped, which resumes an interrupted run.  With
// verbose, a JSON metrics line closes the run.
//
// Host work overlaps the GPU (the reference reads each substack's slices and writes its
// records between its GPU passes, HDoG3D_main.cpp:134-170,246-255): the slices of the next
// stack are read into a second page-locked buffer, and the previous stack's records are
// written from a second record buffer, while the current stack runs.  What a run leaves
// behind is that of a run going stack after stack: a stack's result file is removed only
// after the stack before it was written, whether a stack is skipped is decided after that
// write, and a failing stack (its slices, its GPU work, its write) ends the run after the
// stacks before it were written, with its own error.
extern "C" int hdog_run_param_file(const char *param_path, int verbose) {
  const auto t_start = std::chrono::steady_clock::now();
  hdog_params p;
  std::vector<StackSpec> stacks;
  int file_verbose = 0, skip_existing = 0;
  TRY(load_param_file(param_path, &p, &stacks, &file_verbose, &skip_existing));
  verbose = verbose || file_verbose;
  int margin = 0;
  TRY(validate(&p));
  TRY(hdog_depth_margin(&p, &margin));
  // as many substacks per batch as the longest stack needs, capped to keep memory modest
  int max_len = 0;
  for (auto &s : stacks) max_len = std::max(max_len, (int)s.src.size());
  std::vector<int> z0s;
  TRY(schedule(max_len, p.depth, margin, z0s));
  int max_sub = std::max(1, std::min((int)z0s.size(), 8));
  // the slices some substack of stack i reads (0 when it has no substack), and its substacks
  std::vector<int> last_slice(stacks.size(), 0), n_subs(stacks.size(), 0);
  for (size_t i = 0; i < stacks.size(); i++) {
    const int length = (int)stacks[i].src.size();
    TRY(schedule(length, p.depth, margin, z0s));
    n_subs[i] = (int)z0s.size();
    if (!z0s.empty()) last_slice[i] = std::min(length, z0s.back() + p.depth);
  }
  hdog_ctx *ctx = nullptr;
  TRY(hdog_ctx_create(&p, max_sub, &ctx));
  const int dev = ctx->dev;
  const size_t plane = (size_t)p.width * p.height;
  auto skipped = [&](size_t i) {
    if (!skip_existing) return false;
    if (FILE *e = fopen(stacks[i].dst.c_str(), "rb")) {
      fclose(e);
      return true;
    }
    return false;
  };
  // two page-locked stack buffers (one read from disk while the other runs) and two record
  // buffers (one written to disk while the other fills)
  uint16_t *buf[2] = {nullptr, nullptr};
  size_t cap[2] = {0, 0};
  RecordBuf rbuf[2];
  int rb = 0;
  std::future<SliceRead> pending, writing;
  size_t pending_stack = stacks.size(), writing_stack = 0;
  int pending_slot = 0;
  int64_t n_done = 0, n_skipped = 0, slices = 0, records = 0;
  double read_s = 0.0, wait_s = 0.0;
  auto launch = [](auto &&fn) -> std::future<SliceRead> {
    try {
      return std::async(std::launch::async, fn);
    } catch (...) {   // no thread to spare: the task runs when its result is asked for
      return std::async(std::launch::deferred, fn);
    }
  };
  // starts reading the first stack from `from` on that will not be skipped into buffer
  // `slot` (allocated there first if too small)
  auto prefetch = [&](size_t from, int slot) {
    pending_stack = stacks.size();
    size_t j = from;
    while (j < stacks.size() && (last_slice[j] == 0 || skipped(j))) j++;
    if (j == stacks.size()) return;
    const size_t need = (size_t)last_slice[j] * plane;
    const std::vector<std::string> *src = &stacks[j].src;
    const int last = last_slice[j];
    uint16_t **b = &buf[slot];
    size_t *c = &cap[slot];
    pending = launch([=]() {
      if (need > *c) {
        cudaSetDevice(dev);
        if (*b) cudaFreeHost(*b);
        *b = nullptr;
        *c = 0;
        if (cudaMallocHost(b, need * sizeof(uint16_t)) != cudaSuccess) {
          SliceRead r;
          r.rc = HDOG_ERR_NOMEM;
          r.msg = "pinned host buffer for the stack failed";
          return r;
        }
        *c = need;
      }
      return read_slices(*src, last, *b, plane);
    });
    pending_stack = j;
    pending_slot = slot;
  };
  // waits for the stack being written and counts it
  auto finish_write = [&]() -> int {
    if (!writing.valid()) return HDOG_OK;
    const SliceRead w = writing.get();
    if (w.rc != HDOG_OK) return fail(w.rc, w.msg);
    const size_t k = writing_stack;
    const int64_t n = (int64_t)rbuf[rb ^ 1].n;
    n_done++;
    slices += (int64_t)stacks[k].src.size();
    records += n;
    if (verbose)
      printf("stack %zu: %zu slices, %d substacks, saved count:%lld\n", k, stacks[k].src.size(), n_subs[k],
             (long long)n);
    return HDOG_OK;
  };
  int rc = HDOG_OK;
  prefetch(0, 0);
  for (size_t i = 0; i < stacks.size() && rc == HDOG_OK; i++) {
    const StackSpec &sp = stacks[i];
    if (skipped(i)) {   // a result that exists now still exists after the pending write
      n_skipped++;
      continue;
    }
    if (last_slice[i] == 0) {
      if ((rc = finish_write()) != HDOG_OK) break;
      remove(sp.dst.c_str());
      continue;
    }
    nvtxRangePushA("hdog stack");
    if (pending_stack != i) {
      // the stack ahead was skipped when its read was planned but not now: read it here
      if (pending.valid()) pending.wait();
      prefetch(i, pending_slot);
    }
    const auto t_wait = std::chrono::steady_clock::now();
    const SliceRead got = pending.get();
    wait_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_wait).count();
    read_s += got.seconds;
    const int slot = pending_slot;
    int rc_stack = got.rc;
    if (rc_stack == HDOG_OK) {
      prefetch(i + 1, 1 - slot);   // the next stack's slices land while this one runs
      rbuf[rb].clear();
      std::lock_guard<std::mutex> lock(ctx->mu);
      rc_stack = run_stack_locked(ctx, buf[slot], 0, last_slice[i], rbuf[rb], nullptr);
    }
    const std::string err_stack = rc_stack != HDOG_OK ? (got.rc != HDOG_OK ? got.msg : g_last_error) : "";
    nvtxRangePop();
    // the stack before this one is complete before anything of this one shows
    if ((rc = finish_write()) != HDOG_OK) break;
    if (skipped(i)) {   // the stack before wrote this stack's result path
      n_skipped++;
      continue;
    }
    remove(sp.dst.c_str());
    if (rc_stack != HDOG_OK) {
      rc = fail(rc_stack, err_stack);
      break;
    }
    const hdog_record *rec = rbuf[rb].p;
    const int64_t n = (int64_t)rbuf[rb].n;
    const std::string dst = sp.dst;
    writing = launch([dst, rec, n]() { return write_records(dst, rec, n); });
    writing_stack = i;
    rb ^= 1;
  }
  if (rc == HDOG_OK) rc = finish_write();
  if (writing.valid()) writing.wait();
  if (pending.valid()) pending.wait();   // a read still filling a buffer
  for (uint16_t *b : buf)
    if (b) cudaFreeHost(b);
  for (RecordBuf &r : rbuf) r.release();
  hdog_ctx_destroy(ctx);
  if (verbose) {
    const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    const double vox = (double)slices * (double)plane;
    printf("{\"hdog_main\": {\"status\": %d, \"stacks_done\": %lld, \"stacks_skipped\": %lld, \"slices\": %lld, "
           "\"voxels\": %.0f, \"records\": %lld, \"seconds\": %.3f, \"slice_read_seconds\": %.3f, "
           "\"slice_read_wait_seconds\": %.3f, \"gvox_per_s\": %.3f}}\n",
           rc, (long long)n_done, (long long)n_skipped, (long long)slices, vox, (long long)records, t, read_s,
           wait_s, t > 0 ? vox / t / 1e9 : 0.0);
    fflush(stdout);
  }
  return rc;
}

// ------------------------------------------------------------------ options
extern "C" int hdog_ctx_set_option(hdog_ctx *c, int option, int value) {
  if (!c) return fail(HDOG_ERR_ARG, "null context");
  std::lock_guard<std::mutex> lock(c->mu);
  switch (option) {
    case HDOG_OPT_FUSED_SWEEP: c->use_sweep = value != 0; return HDOG_OK;
    case HDOG_OPT_HOST_BATCH:
      if (value < 0) return fail(HDOG_ERR_ARG, "HDOG_OPT_HOST_BATCH must be >= 0");
      c->host_batch = value;
      return HDOG_OK;
    case HDOG_OPT_WALK_LIMIT:
      if (value < 0) return fail(HDOG_ERR_ARG, "HDOG_OPT_WALK_LIMIT must be >= 0");
      c->walk_limit = value;
      return HDOG_OK;
    default: return fail(HDOG_ERR_ARG, "unknown option");
  }
}

// ------------------------------------------------------------------ diagnostics
extern "C" int hdog_ccl_edge_count(hdog_ctx *c, int64_t *edges, int64_t *capacity) {
  if (!c || !edges || !capacity) return fail(HDOG_ERR_ARG, "hdog_ccl_edge_count: bad argument");
  std::lock_guard<std::mutex> lock(c->mu);
  HDOG_CUDA_TRY(cudaSetDevice(c->dev));
  unsigned long long n = 0;
  HDOG_CUDA_TRY(cudaMemcpy(&n, c->edge_count, sizeof(n), cudaMemcpyDeviceToHost));
  *edges = (int64_t)n;
  *capacity = c->edge_cap;
  return HDOG_OK;
}

// ------------------------------------------------------------------ timing
extern "C" int hdog_timing_enable(hdog_ctx *c, int on) {
  if (!c) return fail(HDOG_ERR_ARG, "null context");
  std::lock_guard<std::mutex> lock(c->mu);
  if (on && !c->timer) c->timer = new EventTimer();
  if (!on && c->timer) {
    delete c->timer;
    c->timer = nullptr;
  }
  return HDOG_OK;
}

extern "C" int hdog_timing_read(hdog_ctx *c, char *buf, size_t cap) {
  if (!c || !buf || cap == 0) return fail(HDOG_ERR_ARG, "hdog_timing_read: bad argument");
  std::lock_guard<std::mutex> lock(c->mu);
  buf[0] = 0;
  if (!c->timer) return HDOG_OK;
  cudaSetDevice(c->dev);
  c->timer->collect();
  std::string out;
  for (auto &t : c->timer->totals) {
    char line[256];
    snprintf(line, sizeof(line), "%s %lld %.6f\n", t.first.c_str(), (long long)t.second.count, t.second.ms);
    out += line;
  }
  c->timer->totals.clear();
  if (out.size() + 1 > cap) return fail(HDOG_ERR_CAPACITY, "timing buffer too small");
  memcpy(buf, out.c_str(), out.size() + 1);
  return HDOG_OK;
}

// ------------------------------------------------------------------ helpers
extern "C" int hdog_memcpy(void *dst, const void *src, size_t bytes, void *stream) {
  if (bytes == 0) return HDOG_OK;
  if (!dst || !src) return fail(HDOG_ERR_ARG, "hdog_memcpy: null pointer");
  HDOG_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream));
  HDOG_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return HDOG_OK;
}
extern "C" int hdog_stream_sync(void *stream) {
  HDOG_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return HDOG_OK;
}
extern "C" int hdog_device_alloc(void **ptr, size_t bytes) {
  if (!ptr) return fail(HDOG_ERR_ARG, "hdog_device_alloc: null pointer");
  HDOG_CUDA_TRY(cudaMalloc(ptr, bytes));
  return HDOG_OK;
}
extern "C" int hdog_device_free(void *ptr) {
  HDOG_CUDA_TRY(cudaFree(ptr));
  return HDOG_OK;
}
