// kernels.cuh -- substack descriptors and the launchers each .cu file exports.
#pragma once
#include "common.cuh"

namespace hdog {

// One substack of a batch.  Volume arrays of a batch hold the substacks back to back;
// substack s starts at voxel offset `vox`.  Kernels take the descriptor array in device
// memory and use blockIdx.y as the substack index, blockIdx.x as the tile index inside
// it (blocks past a smaller substack's tile count return at once).
struct Sub {
  int W, H, D;            // extent; D = HDoG_param.depth
  int depth_valid;        // slices read from `src`; slices >= depth_valid are zero
  int z0;                 // global z of slice 0, added to record centroid_z
  int margin;             // depth margin m (records keep m <= cz < depth_valid - m)
  int64_t vox;            // voxel offset of this substack in the batch volume arrays
  int64_t reg;            // offset of its region slots in the region arrays
  int64_t reg_cap;        // number of region slots (background included)
  int64_t blk;            // offset of its per-block slots in block scratch arrays
  int64_t edge;           // offset of its cross-tile edge list
  int64_t edge_cap;       // edge list capacity
  int64_t fg;             // offset of its foreground list (fused DoG/Hessian sweep)
  int64_t fg_cap;         // foreground list capacity
  const uint16_t *src;    // slice 0 of the raw input (device); slices are W*H apart
  int64_t walk_limit;     // bound of the labelling's union-find walks and retries (0: W*H*D)
};

// A device work queue of (substack, tile) items for a persistent launch: item i is tile
// i % tiles of substack i / tiles; blocks take items with atomicAdd on *next (zeroed before
// the launch) until it passes total.
struct WorkQueue {
  unsigned *next;
  int total;
  int tiles;
};

// Launch shape of the sweeps: blocks per SM of a persistent launch over the work queue, or
// 0 for one block per tile and substack.  Chosen per frame shape by the autotuner.
struct LaunchShape {
  int dog_per_sm = 0;
  int hess_per_sm = 0;
  int num_sms = 152;
};

// Foreground-list counters of the substacks of a batch sit kFgCountStride 64-bit slots
// apart: every warp of the Hessian sweep takes its list slots with an atomic on its
// substack's counter, and counters on separate 4 KB lines spread those atomics over L2.
constexpr int kFgCountStride = 512;

// A foreground voxel and its six Hessian elements, written by the fused sweep.
struct FgEntry {
  int32_t idx;            // linear voxel index inside the substack
  float norm;             // normalized intensity at the voxel
  float h[6];             // xx, xy, xz, yy, yz, zz
};

// Per-region accumulators (SoA over all region slots of a batch).
struct RegionAcc {
  int32_t *label;         // root voxel index (local to the substack)
  uint32_t *count;
  uint32_t *max_ord;      // f2ord(max normalized intensity)
  unsigned long long *sum_xyz;   // [3][cap] exact coordinate sums
  unsigned long long *sum_norm;  // fixed point (kFixScale)
  unsigned long long *hess;      // [6][cap] fixed point (kFixScale)
};

struct RegionOut {
  float *intensity;       // [cap]
  float *centroid;        // [3][cap]
  float *hessian;         // [6][cap]
  float *eigen;           // [2][cap]
  uint8_t *keep;          // [cap] record filter result
};

struct FilterParams {
  int left, right, top, bottom;
  int min_size;
  int is_ave_mode;
  int all_eigen;          // eigen features for every region, not only the kept ones
};

inline unsigned ceil_div(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// ---- norm.cu ----
// ma, mb: packed u32 volumes; fa, fb: float2 volumes (ma/mb may alias fb's two halves).
// src_aligned8: every substack's src is 8-byte aligned (four-column z loads).
// ero_l, dil_l (optional): also write the box means of the min and the max.
void launch_normalize(const Sub *d_subs, int nsub, int W, int H, int D, int rxy, int rz, float min_intensity,
                      bool src_aligned8, uint32_t *ma, uint32_t *mb, float2 *fa, float2 *fb, float *norm,
                      cudaStream_t s, float *ero_l = nullptr, float *dil_l = nullptr);
void launch_copy_norm(const Sub *d_subs, int nsub, int64_t max_n, float min_intensity,
                      float *norm, cudaStream_t s);
// tmp: two packed u32 volumes of nsub substacks each; dst: uint16 (substack s at S.vox).
void launch_erosion(const Sub *d_subs, int nsub, int W, int H, int D, int rxy, int rz, bool src_aligned8,
                    uint32_t *tmp, uint16_t *dst, cudaStream_t s);
// ---- dog.cu ----
void launch_dog(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, int64_t max_rows,
                const DogTaps &T, const float *norm, float2 *t0, float2 *t1, float *dog, cudaStream_t s);
void launch_hessian_pd(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d,
                       const float *dog, uint8_t *mask, float *hess6, cudaStream_t s);
// ---- sweep.cu ----
constexpr int kMaxSweepRxy = 12;
size_t sweep_smem_bytes(int rxy);
bool sweep_supported(const DogTaps &T, int W, int max_smem);
// DoG volume by the radius-specialised z-sweep; false (nothing launched) when the radii
// have no instantiation or the buffers do not suit TMA.
// records.cu: per-record steps after the records (host-side NumPy in the reference)
void launch_to_global(const hdog_record *rec, int64_t n, const hdog_global_params &p, hdog_global *out,
                      cudaStream_t s);
void launch_scale_merge(const hdog_global *in, int64_t n, const hdog_scalemerge_params &p, hdog_scalemerged *out,
                        cudaStream_t s);
void launch_clf_features(const hdog_record *rec, int64_t n, const hdog_clf_params &p, double *X, cudaStream_t s);

// soft.cu: the differentiable chain (hdog_soft_*); status codes as the C ABI
size_t soft_workspace_bytes(const hdog_soft_params &p);
int soft_forward(const hdog_soft_params *p, const float *vol, const int32_t *pos, int n_pos, const int32_t *neg,
                 int n_neg, float *loss, float *scores, void *work, cudaStream_t st);
int soft_backward(const hdog_soft_params *p, const float *vol, const int32_t *pos, int n_pos, const int32_t *neg,
                  int n_neg, float grad_loss, float *grad_vol, float *grad_sigma, float *grad_thresh, void *work,
                  cudaStream_t st, bool forward_kept = false);

// Zero `bytes` (a multiple of 4) of device memory on stream s with a kernel.
void zero_async(void *p, size_t bytes, cudaStream_t s);
void pack_fg_counts_async(const unsigned long long *fg_count, int nsub, unsigned long long *packed, cudaStream_t s);

bool launch_dog_sweep(const Sub *d_subs, int nsub, int W, int H, int D, const DogTaps &T, const float *norm,
                      float *dog, int *d_status, int max_smem, cudaStream_t s);
// DoG + Hessian + PD: the radius-specialised pair (norm -> dog -> mask + list) when the tap
// radii have an instantiation, else the generic fused sweep (dog untouched).
// ls / qctr (two device counters): the launch shape of the radius-specialised sweeps.
int launch_dog_hess(const Sub *d_subs, int nsub, int W, int H, int D, const DogTaps &T, const float *norm,
                    float *dog, uint8_t *mask, FgEntry *fg, int32_t *fg_idx, unsigned long long *fg_count,
                    int *d_status, const LaunchShape &ls, unsigned *qctr, cudaStream_t s);
// ---- ccl.cu ----
// Segments of a per-substack scan: substack s scans len[s] counts starting at off[s];
// chk[s] is its offset in the chunk-sum scratch (one slot per 1024 counts).
struct ScanSeg {
  const int64_t *off, *len, *chk;
  int64_t max_len;
};
void launch_scan(const ScanSeg &sg, int nsub, const uint32_t *in, uint32_t *out, uint32_t *chunk,
                 int64_t *totals, int64_t add, cudaStream_t s);
void launch_ccl(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, int64_t max_n, const uint8_t *mask,
                int32_t *labels, int2 *edges, unsigned long long *edge_count, uint32_t *root_bits,
                uint32_t *blk_counts, int *d_status, int num_sms, cudaStream_t s, const FgEntry *fg = nullptr,
                const unsigned long long *fg_count = nullptr, int64_t max_fg = 0, int64_t nblk = 0,
                int32_t *fg_root = nullptr);
// Foreground mask (label != 0), root bitmap and per-block root counts from labels alone.
void launch_roots_from_labels(const Sub *d_subs, int nsub, int64_t max_n, const int32_t *labels, uint8_t *mask,
                              uint32_t *root_bits, uint32_t *blk_counts, cudaStream_t s);
void launch_regions(const Sub *d_subs, int nsub, int64_t max_n, const ScanSeg &vseg, const uint8_t *mask,
                    const int32_t *labels, const uint32_t *root_bits, const float *norm, const float *dog,
                    int32_t *rank, uint32_t *blk_counts, uint32_t *blk_offsets, uint32_t *chunk,
                    int64_t *d_num_regions, RegionAcc acc, int64_t slots, int *d_status, cudaStream_t s);
// Accumulation from the fused sweep's foreground list instead of the mask and DoG.
void launch_regions_fg(const Sub *d_subs, int nsub, int64_t max_n, int64_t max_fg, const ScanSeg &vseg,
                       const int32_t *fg_root, const uint32_t *root_bits, const FgEntry *fg,
                       const unsigned long long *fg_count, int32_t *rank, uint32_t *blk_counts,
                       uint32_t *blk_offsets, uint32_t *chunk, int64_t *d_num_regions, RegionAcc acc, int64_t slots,
                       int *d_status, int num_sms, cudaStream_t s);
void launch_finalize(const Sub *d_subs, int nsub, int64_t max_reg_cap, const ScanSeg &rseg,
                     const int64_t *d_num_regions, RegionAcc acc, int64_t slots, RegionOut out,
                     FilterParams fp, uint32_t *blk_counts, uint32_t *blk_offsets, uint32_t *chunk,
                     int64_t *d_num_records, hdog_record *records, int64_t blk_stride, cudaStream_t s);

// ---- graph.cu: record placement of the batched graph form ----
constexpr int kGraphMaxBatch = 64;   // substacks per batch in the graph form
struct GraphIds {
  int id[kGraphMaxBatch];            // the run's index of each batch substack
};
struct GraphSlot {
  long long off, count;              // a substack's records in the run's record array
};
void launch_graph_place(int nsub, const GraphIds &ids, const int64_t *num_records, const unsigned long long *fg_count,
                        int64_t fg_cap, bool fused, const int *status, int64_t *total, GraphSlot *table, int *redo,
                        int64_t out_cap, cudaStream_t s);
void launch_graph_copy(int nsub, const GraphIds &ids, const hdog_record *records, int64_t reg_cap,
                       const GraphSlot *table, hdog_record *out, int64_t out_cap, cudaStream_t s);

constexpr int kMaxRadiusXY = 421;    // shared-memory bound of the min/max x and y passes
constexpr int kScanBlock = 4096;     // voxels per block in the region scans (16 per thread)
constexpr int kFinalizeBlock = 256;  // regions per block in finalize / record compaction

}  // namespace hdog
