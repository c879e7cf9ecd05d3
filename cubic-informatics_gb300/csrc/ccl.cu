// ccl.cu -- 3D connected-component labelling with the reference's connectivity, sm_103a.
//
// Reference: src/3D/CCL3D.cu (CCL :81-117).  The reference iterates neighbour-min scans
// and pointer jumping, synchronising with the host twice per iteration.  Its fixed point
// labels each component with the minimum linear index of its voxels, over a graph whose
// edges are the 26 LINEAR offsets dz*W*H + dy*W + dx kept inside [0, N) -- so a row end
// touches the next row's start and a slice's last row the next slice's first -- and in
// which voxel 0 is background (label = index * mask).
//
// Here the same labels come from union-find in three passes, with no host round trip:
//   1. k_ccl_local: a 64 x 16 x 32 tile (a whole 32-slice substack column) is labelled in
//      shared memory with 16-bit parents; the tile's foreground edges that leave the
//      tile (its x and y faces, and the wrap-around offsets) go to a compact edge list.
//   2. k_ccl_edges: a persistent pass merges those edges in the global label array.
//      If the list overflowed, k_ccl_cross_direct merges the same edges from the mask.
//   3. k_ccl_flatten: every foreground voxel gets its root (a read-only walk, so every
//      store is final); roots are recorded in a bitmap and counted per 4096 voxels for
//      the region numbering.
// Linking always hangs the larger root under the smaller, so roots are component minima.
#include "kernels.cuh"

namespace hdog {

// ------------------------------------------------------------------ global union-find
// Invariants: a parent pointer only ever points to a smaller index in the same tree; a
// root is linked only by a compare-and-swap that requires it to still be a root, so
// trees merge but never split.  A stale read (the L1 cache is not coherent across SMs)
// can then only show an older pointer of the same tree: two finds that meet at one node
// are truly in one tree, and a link attempted on a former root fails and retries from
// its current parent.  Path halving stores only an ancestor of the node's parent.
__device__ __forceinline__ int32_t uf_find(int32_t *L, int32_t a, int64_t limit, int *status) {
  int32_t p = __ldcg(L + a);
  int64_t steps = 0;
  while (p != a) {
    const int32_t gp = __ldcg(L + p);
    if (gp != p) L[a] = gp;
    a = p;
    p = gp;
    if (++steps > limit) { atomicExch(status, HDOG_ERR_TIMEOUT); break; }
  }
  return a;
}

// Read-only walk, for the flatten pass where every store must be a final root.
__device__ __forceinline__ int32_t uf_root(const int32_t *L, int32_t a, int64_t limit, int *status) {
  int32_t p = __ldcg(L + a);
  int64_t steps = 0;
  while (p != a) {
    a = p;
    p = __ldcg(L + a);
    if (++steps > limit) { atomicExch(status, HDOG_ERR_TIMEOUT); break; }
  }
  return a;
}

__device__ __forceinline__ void uf_union(int32_t *L, int32_t a, int32_t b, int64_t limit, int *status) {
  for (int64_t it = 0; it <= limit; it++) {
    a = uf_find(L, a, limit, status);
    b = uf_find(L, b, limit, status);
    if (a == b) return;
    if (a > b) { const int32_t t = a; a = b; b = t; }
    const int32_t cur = atomicCAS(&L[b], b, a);
    if (cur == b) return;
    b = cur;
  }
  atomicExch(status, HDOG_ERR_TIMEOUT);
}

// The 13 backward linear offsets (the other 13 of the 26 are their mirror images).
__device__ __forceinline__ void back_offset(int k, int &dz, int &dy, int &dx) {
  dz = k < 9 ? -1 : 0;
  dy = k < 9 ? k / 3 - 1 : (k < 12 ? -1 : 0);
  dx = k < 9 ? k % 3 - 1 : (k < 12 ? k - 10 : -1);
}

// ------------------------------------------------------------------ pass 1: tile-local
constexpr int kTX = 64, kTY = 16, kTZ = 32;
constexpr int kTileVox = kTX * kTY * kTZ;     // 32768: parents fit in 16 bits
constexpr int kCclThreads = 256;              // thread = 4 x-consecutive voxels of one row, all kTZ slices
constexpr uint16_t kBg = 0xFFFF;

// Find with path halving (stores an ancestor of the parent only, as in the global
// version); without it "smaller root wins" linking grows long chains.
__device__ __forceinline__ int sfind(volatile uint16_t *lab, int t) {
  int p = lab[t];
  while (p != t) {
    const int gp = lab[p];
    if (gp != p) lab[t] = (uint16_t)gp;
    t = p;
    p = gp;
  }
  return t;
}

// Read-only find for the final pass over a finished forest.
__device__ __forceinline__ int sroot(const uint16_t *lab, int t) {
  int p = lab[t];
  while (p != t) {
    t = p;
    p = lab[t];
  }
  return t;
}

__device__ __forceinline__ void sunion(uint16_t *lab, int a, int b) {
  volatile uint16_t *v = lab;
  for (int it = 0; it < 2 * kTileVox; it++) {
    a = sfind(v, a);
    b = sfind(v, b);
    if (a == b) return;
    if (a > b) { const int t = a; a = b; b = t; }
    const unsigned short cur = atomicCAS(reinterpret_cast<unsigned short *>(&lab[b]), (unsigned short)b,
                                         (unsigned short)a);
    if (cur == b) return;
    b = cur;
  }
}

struct CclTile {
  int x0, y0, z0, tz;     // origin, slices in this tile
};

__device__ __forceinline__ bool ccl_tile(const Sub &S, int64_t bid, CclTile &T) {
  const int nx = (S.W + kTX - 1) / kTX, ny = (S.H + kTY - 1) / kTY, nz = (S.D + kTZ - 1) / kTZ;
  if (bid >= (int64_t)nx * ny * nz) return false;
  T.x0 = (int)(bid % nx) * kTX;
  T.y0 = (int)((bid / nx) % ny) * kTY;
  T.z0 = (int)(bid / ((int64_t)nx * ny)) * kTZ;
  T.tz = min(kTZ, S.D - T.z0);
  return true;
}

// Backward neighbour (dz, dy, dx) of voxel (x, y, z), tile coordinates (lx, ly, lz):
// true when the edge is not a plain 3D step inside this tile (it leaves the tile, or
// it wraps around a row or slice end).
__device__ __forceinline__ bool leaves_tile(const Sub &S, const CclTile &T, int x, int y, int z, int lx, int ly,
                                            int lz, int dz, int dy, int dx) {
  const int nx = x + dx, ny = y + dy, nz = z + dz;
  const bool in_vol = nx >= 0 && nx < S.W && ny >= 0 && ny < S.H && nz >= 0;
  const bool in_tile = lx + dx >= 0 && lx + dx < kTX && ly + dy >= 0 && ly + dy < kTY && lz + dz >= 0 && lz + dz < T.tz;
  return !(in_vol && in_tile);
}

constexpr int kFgList = 12288;                // compact foreground list of a tile (37.5%)

__device__ __forceinline__ uint32_t tile_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t ws[kCclThreads / 32 + 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t inc = v;
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, d);
    if (lane >= d) inc += y;
  }
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int k = 0; k < kCclThreads / 32; k++) { const uint32_t c = ws[k]; ws[k] = run; run += c; }
    ws[kCclThreads / 32] = run;
  }
  __syncthreads();
  const uint32_t r = ws[w] + inc - v;
  *total = ws[kCclThreads / 32];
  __syncthreads();
  return r;
}

// Union of tile voxel lt with its backward neighbours inside the tile; counts the
// foreground edges that leave the tile and, when `emit`, writes them from slot *base.
__device__ __forceinline__ int tile_voxel_edges(const Sub &S, const CclTile &T, uint16_t *lab, const uint8_t *m,
                                                int lt, bool do_union, bool emit, int2 *edges,
                                                unsigned long long *base) {
  const int lx = lt % kTX, ly = (lt / kTX) % kTY, lz = lt / (kTX * kTY);
  const int x = T.x0 + lx, y = T.y0 + ly, z = T.z0 + lz;
  const int64_t WH = (int64_t)S.W * S.H;
  const int64_t g = z * WH + (int64_t)y * S.W + x;
  int n_cross = 0;
  for (int o = 0; o < 13; o++) {
    int dz, dy, dx;
    back_offset(o, dz, dy, dx);
    if (!leaves_tile(S, T, x, y, z, lx, ly, lz, dz, dy, dx)) {
      if (!do_union) continue;
      const int ln = lt + (dz * kTY + dy) * kTX + dx;
      const uint16_t pn = lab[ln];
      if (pn != kBg && pn != lab[lt]) sunion(lab, lt, ln);
    } else {
      const int64_t gn = g + dz * WH + dy * (int64_t)S.W + dx;
      if (gn >= 1 && m[gn]) {
        if (emit) {
          if ((int64_t)*base < S.edge_cap) edges[S.edge + *base] = make_int2((int32_t)g, (int32_t)gn);
          (*base)++;
        }
        n_cross++;
      }
    }
  }
  return n_cross;
}

__global__ void __launch_bounds__(kCclThreads) k_ccl_local(const Sub *subs, const uint8_t *mask, int32_t *labels,
                                                          int2 *edges, unsigned long long *edge_count) {
  extern __shared__ uint16_t lab[];   // kTileVox parents, then kFgList foreground indices
  uint16_t *fgl = lab + kTileVox;
  const Sub S = subs[blockIdx.y];
  CclTile T;
  if (!ccl_tile(S, blockIdx.x, T)) return;
  const int t = threadIdx.x;
  const int lx0 = (t % (kTX / 4)) * 4, ly = t / (kTX / 4);
  const int x = T.x0 + lx0, y = T.y0 + ly;
  const int64_t WH = (int64_t)S.W * S.H;
  const uint8_t *m = mask + S.vox;
  const bool row_ok = y < S.H;
  const bool vec = row_ok && x + 3 < S.W && (S.W % 4 == 0) &&
                   ((reinterpret_cast<uintptr_t>(m + (int64_t)y * S.W + x) & 3) == 0);
  // 1. foreground -> own tile index, background -> kBg; count this thread's foreground
  uint32_t nfg = 0;
  for (int lz = 0; lz < kTZ; lz++) {
    const int lt = (lz * kTY + ly) * kTX + lx0;
    uint32_t w = 0;
    if (lz < T.tz) {
      const int64_t g = (T.z0 + lz) * WH + (int64_t)y * S.W + x;
      if (vec) {
        w = __ldg(reinterpret_cast<const uint32_t *>(m + g));
      } else if (row_ok) {
        for (int k = 0; k < 4; k++)
          if (x + k < S.W && m[g + k]) w |= 0xFFu << (8 * k);
      }
      if (g == 0) w &= ~0xFFu;   // voxel 0 is background
    }
    ushort4 v;
    v.x = (w & 0xFFu) ? (uint16_t)lt : kBg;
    v.y = ((w >> 8) & 0xFFu) ? (uint16_t)(lt + 1) : kBg;
    v.z = ((w >> 16) & 0xFFu) ? (uint16_t)(lt + 2) : kBg;
    v.w = (w >> 24) ? (uint16_t)(lt + 3) : kBg;
    nfg += (v.x != kBg) + (v.y != kBg) + (v.z != kBg) + (v.w != kBg);
    *reinterpret_cast<ushort4 *>(&lab[lt]) = v;
  }
  // 2. compact list of foreground tile indices (block scan of the per-thread counts)
  uint32_t total;
  const uint32_t off = tile_scan(nfg, &total);
  const bool listed = total <= (uint32_t)kFgList;
  if (listed) {
    uint32_t o = off;
    for (int lz = 0; lz < T.tz; lz++)
      for (int k = 0; k < 4; k++) {
        const int lt = (lz * kTY + ly) * kTX + lx0 + k;
        if (lab[lt] != kBg) fgl[o++] = (uint16_t)lt;
      }
  }
  __syncthreads();
  // 3. unions inside the tile, foreground voxels spread evenly over the threads
  int n_cross = 0;
  if (listed) {
    for (uint32_t i = t; i < total; i += kCclThreads)
      n_cross += tile_voxel_edges(S, T, lab, m, fgl[i], true, false, nullptr, nullptr);
  } else {
    for (int lz = 0; lz < T.tz; lz++)
      for (int k = 0; k < 4; k++) {
        const int lt = (lz * kTY + ly) * kTX + lx0 + k;
        if (lab[lt] != kBg) n_cross += tile_voxel_edges(S, T, lab, m, lt, true, false, nullptr, nullptr);
      }
  }
  __syncthreads();
  // 4. final roots stored in place (no union runs any more, so only roots are stored)
  if (listed) {
    for (uint32_t i = t; i < total; i += kCclThreads) lab[fgl[i]] = (uint16_t)sroot(lab, fgl[i]);
  } else {
    for (int lz = 0; lz < T.tz; lz++)
      for (int k = 0; k < 4; k++) {
        const int lt = (lz * kTY + ly) * kTX + lx0 + k;
        if (lab[lt] != kBg) lab[lt] = (uint16_t)sroot(lab, lt);
      }
  }
  // 5. reserve edge slots (one atomic per warp) and emit the edges in the same order
  const int lane = threadIdx.x & 31;
  int incl = n_cross;
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if (lane >= d) incl += v;
  }
  const int warp_total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  unsigned long long base = 0;
  if (lane == 31 && warp_total) base = atomicAdd(&edge_count[blockIdx.y], (unsigned long long)warp_total);
  base = __shfl_sync(0xFFFFFFFFu, base, 31) + (unsigned long long)(incl - n_cross);
  if (n_cross) {
    if (listed) {
      for (uint32_t i = t; i < total; i += kCclThreads)
        tile_voxel_edges(S, T, lab, m, fgl[i], false, true, edges, &base);
    } else {
      for (int lz = 0; lz < T.tz; lz++)
        for (int k = 0; k < 4; k++) {
          const int lt = (lz * kTY + ly) * kTX + lx0 + k;
          if (lab[lt] != kBg) tile_voxel_edges(S, T, lab, m, lt, false, true, edges, &base);
        }
    }
  }
  __syncthreads();
  // 6. labels: tile root -> its global index, background -> 0 (whole rows, vector stores)
  if (!row_ok) return;
  int32_t *L = labels + S.vox;
  for (int lz = 0; lz < T.tz; lz++) {
    const int64_t g = (T.z0 + lz) * WH + (int64_t)y * S.W + x;
    const ushort4 v = *reinterpret_cast<const ushort4 *>(&lab[(lz * kTY + ly) * kTX + lx0]);
    const uint16_t r4[4] = {v.x, v.y, v.z, v.w};
    int32_t out[4];
    for (int k = 0; k < 4; k++) {
      const int r = r4[k];
      out[k] = r == kBg ? 0
                        : (int32_t)((T.z0 + r / (kTX * kTY)) * WH + (int64_t)(T.y0 + (r / kTX) % kTY) * S.W + T.x0 +
                                    r % kTX);
    }
    if (vec) {
      *reinterpret_cast<int4 *>(L + g) = make_int4(out[0], out[1], out[2], out[3]);
    } else {
      for (int k = 0; k < 4; k++)
        if (x + k < S.W) L[g + k] = out[k];
    }
  }
}

// ------------------------------------------------------------------ pass 2: cross-tile edges
__global__ void k_ccl_edges(const Sub *subs, const int2 *edges, const unsigned long long *edge_count,
                            int32_t *labels, int *status) {
  const Sub S = subs[blockIdx.y];
  const unsigned long long cnt = edge_count[blockIdx.y];
  if (cnt > (unsigned long long)S.edge_cap) return;   // overflowed: k_ccl_cross_direct merges instead
  const int64_t n = (int64_t)S.W * S.H * S.D;
  int32_t *L = labels + S.vox;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)cnt;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int2 ab = edges[S.edge + e];
    uf_union(L, ab.x, ab.y, n, status);
  }
}

// The same cross-tile edges straight from the mask, for a substack whose list overflowed.
__global__ void __launch_bounds__(kCclThreads) k_ccl_cross_direct(const Sub *subs, const uint8_t *mask,
                                                                 const unsigned long long *edge_count,
                                                                 int32_t *labels, int *status) {
  const Sub S = subs[blockIdx.y];
  if (edge_count[blockIdx.y] <= (unsigned long long)S.edge_cap) return;
  CclTile T;
  if (!ccl_tile(S, blockIdx.x, T)) return;
  const int t = threadIdx.x;
  const int lx0 = (t % (kTX / 4)) * 4, ly = t / (kTX / 4);
  const int x = T.x0 + lx0, y = T.y0 + ly;
  if (y >= S.H) return;
  const int64_t WH = (int64_t)S.W * S.H, n = WH * S.D;
  const uint8_t *m = mask + S.vox;
  int32_t *L = labels + S.vox;
  for (int lz = 0; lz < T.tz; lz++) {
    const int z = T.z0 + lz;
    for (int k = 0; k < 4 && x + k < S.W; k++) {
      const int64_t g = z * WH + (int64_t)y * S.W + x + k;
      if (g == 0 || !m[g]) continue;
      for (int o = 0; o < 13; o++) {
        int dz, dy, dx;
        back_offset(o, dz, dy, dx);
        if (!leaves_tile(S, T, x + k, y, z, lx0 + k, ly, lz, dz, dy, dx)) continue;
        const int64_t gn = g + dz * WH + dy * (int64_t)S.W + dx;
        if (gn >= 1 && m[gn]) uf_union(L, (int32_t)g, (int32_t)gn, n, status);
      }
    }
  }
}

// ------------------------------------------------------------------ pass 3: flatten
// 4096 voxels per block, 16 consecutive voxels per thread.  Root bits of voxels
// [32w, 32w+32) of block b go to word (S.blk + b) * 128 + w.
template <bool FROM_LABELS>
__global__ void __launch_bounds__(256) k_ccl_flatten(const Sub *subs, uint8_t *mask, int32_t *labels,
                                                    uint32_t *root_bits, uint32_t *blk_counts, int *status) {
  __shared__ uint32_t wcnt[8];
  const Sub S = subs[blockIdx.y];
  const int64_t n = (int64_t)S.W * S.H * S.D;
  const int64_t base = (int64_t)blockIdx.x * kScanBlock;
  if (base >= n) return;
  const int64_t i0 = base + threadIdx.x * 16;
  int32_t *L = labels + S.vox;
  uint8_t *m = mask + S.vox;
  uint32_t bits = 0;
  if (!FROM_LABELS) {
    uint8_t mk[16];
    if (i0 + 16 <= n && ((reinterpret_cast<uintptr_t>(m + i0) & 15) == 0)) {
      *reinterpret_cast<uint4 *>(mk) = __ldg(reinterpret_cast<const uint4 *>(m + i0));
    } else {
      for (int k = 0; k < 16; k++) mk[k] = (i0 + k < n) ? m[i0 + k] : 0;
    }
    for (int k = 0; k < 16; k++) {
      const int64_t i = i0 + k;
      if (i == 0 || !mk[k]) continue;
      const int32_t l = __ldcg(L + i);
      const int32_t r = uf_root(L, l, n, status);
      if (r != l) L[i] = r;
      if (r == (int32_t)i) bits |= 1u << k;
    }
  } else {
    // labels produced elsewhere: foreground = nonzero label, roots label themselves
    for (int k = 0; k < 16; k++) {
      const int64_t i = i0 + k;
      if (i >= n) break;
      const int32_t l = L[i];
      m[i] = l != 0;
      if (i > 0 && l == (int32_t)i) bits |= 1u << k;
    }
  }
  const uint32_t hi = __shfl_down_sync(0xFFFFFFFFu, bits, 1);
  if ((threadIdx.x & 1) == 0) root_bits[(S.blk + blockIdx.x) * (kScanBlock / 32) + threadIdx.x / 2] = bits | (hi << 16);
  uint32_t c = __popc(bits);
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
  if ((threadIdx.x & 31) == 0) wcnt[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int k = 0; k < 8; k++) tot += wcnt[k];
    blk_counts[S.blk + blockIdx.x] = tot;
  }
}

// ------------------------------------------------------------------ launchers
void launch_ccl(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, int64_t max_n, const uint8_t *mask,
                int32_t *labels, int2 *edges, unsigned long long *edge_count, uint32_t *root_bits,
                uint32_t *blk_counts, int *d_status, int num_sms, cudaStream_t s) {
  const int64_t tiles = (int64_t)ceil_div(max_w, kTX) * ceil_div(max_h, kTY) * ceil_div(max_d, kTZ);
  cudaMemsetAsync(edge_count, 0, nsub * sizeof(unsigned long long), s);
  const int smem = (kTileVox + kFgList) * (int)sizeof(uint16_t);
  cudaFuncSetAttribute(k_ccl_local, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  KLAUNCH("k_ccl_local", s, (k_ccl_local<<<dim3((unsigned)tiles, nsub), kCclThreads, smem, s>>>(
                                d_subs, mask, labels, edges, edge_count)));
  const unsigned eb = (unsigned)max(1, (8 * num_sms + nsub - 1) / nsub);
  KLAUNCH("k_ccl_edges", s, (k_ccl_edges<<<dim3(eb, nsub), 256, 0, s>>>(d_subs, edges, edge_count, labels,
                                                                        d_status)));
  KLAUNCH("k_ccl_cross_direct", s, (k_ccl_cross_direct<<<dim3((unsigned)tiles, nsub), kCclThreads, 0, s>>>(
                                       d_subs, mask, edge_count, labels, d_status)));
  KLAUNCH("k_ccl_flatten", s, (k_ccl_flatten<false><<<dim3(ceil_div(max_n, kScanBlock), nsub), 256, 0, s>>>(
                                  d_subs, const_cast<uint8_t *>(mask), labels, root_bits, blk_counts, d_status)));
}

void launch_roots_from_labels(const Sub *d_subs, int nsub, int64_t max_n, const int32_t *labels, uint8_t *mask,
                              uint32_t *root_bits, uint32_t *blk_counts, cudaStream_t s) {
  KLAUNCH("k_roots_from_labels", s, (k_ccl_flatten<true><<<dim3(ceil_div(max_n, kScanBlock), nsub), 256, 0, s>>>(
                                        d_subs, mask, const_cast<int32_t *>(labels), root_bits, blk_counts,
                                        nullptr)));
}

}  // namespace hdog
