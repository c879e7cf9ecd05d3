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
//      shared memory over its 2 x 2 x 2 cells (see below); the foreground edges that
//      leave the tile (its x and y faces, and the wrap-around offsets) go to an edge list.
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
constexpr int kTileVox = kTX * kTY * kTZ;     // 32768 voxels
constexpr int kCclThreads = 256;              // thread = 4 x-consecutive voxels of one row, all kTZ slices

// Shared-memory union-find over the tile's cells, 32-bit parents (native shared atomics;
// kBg32 marks a background cell).  Find with path halving (stores an ancestor of the
// parent only, as in the global version); without it "smaller root wins" linking grows
// long chains.
constexpr uint32_t kBg32 = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t sfind(volatile uint32_t *par, uint32_t t) {
  uint32_t p = par[t];
  while (p != t) {
    const uint32_t gp = par[p];
    if (gp != p) par[t] = gp;
    t = p;
    p = gp;
  }
  return t;
}

// Read-only find for the final pass over a finished forest.
__device__ __forceinline__ uint32_t sroot(const uint32_t *par, uint32_t t) {
  uint32_t p = par[t];
  while (p != t) {
    t = p;
    p = par[t];
  }
  return t;
}

__device__ __forceinline__ void sunion(uint32_t *par, uint32_t a, uint32_t b, uint32_t limit) {
  volatile uint32_t *v = par;
  for (uint32_t it = 0; it < limit; it++) {
    a = sfind(v, a);
    b = sfind(v, b);
    if (a == b) return;
    if (a > b) { const uint32_t t = a; a = b; b = t; }
    const uint32_t cur = atomicCAS(&par[b], b, a);
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

constexpr int kEdgeBuf = 2048;                // cross-tile edges staged per tile before one global reservation

// ---- cell union-find inside the tile
// Inside a tile every edge is a plain 26-neighbour step (the reference's row and slice
// wrap-arounds always leave the tile and go to the edge list), and any two foreground
// voxels of one 2 x 2 x 2 cell are 26-neighbours.  So the tile is labelled over cells:
// a cell is one union-find node, its 8-bit occupancy says which voxels are foreground
// (bit 4*dz + 2*dy + dx, i.e. linear voxel order), and two neighbouring cells are
// connected exactly when each has a foreground voxel on the side facing the other --
// two mask tests per pair.  A component's label is then the minimum voxel index over
// its cells, found with one shared-memory atomicMin per cell.
constexpr int kCX = kTX / 2, kCY = kTY / 2, kCZ = kTZ / 2;
constexpr int kCells = kCX * kCY * kCZ;       // 4096

// Occupancy bits of a cell whose voxels have local coordinate `side` along one axis
// (0 or 1); axis 0 = x, 1 = y, 2 = z.
__host__ __device__ constexpr uint8_t cell_side(int axis, int side) {
  uint8_t m = 0;
  for (int v = 0; v < 8; v++)
    if (((v >> axis) & 1) == side) m |= (uint8_t)(1u << v);
  return m;
}
// For cell offset d (-1, 0, +1) along an axis: the voxels of this cell (self) and of the
// neighbour that can touch across it.
__host__ __device__ constexpr uint8_t cell_face(int axis, int d, bool self) {
  return d == 0 ? (uint8_t)0xFF : (d < 0 ? cell_side(axis, self ? 0 : 1) : cell_side(axis, self ? 1 : 0));
}
struct CellNb {
  int dz, dy, dx;
  uint8_t self, other;
};
__host__ __device__ constexpr CellNb cell_nb(int dz, int dy, int dx) {
  return CellNb{dz, dy, dx,
                (uint8_t)(cell_face(0, dx, true) & cell_face(1, dy, true) & cell_face(2, dz, true)),
                (uint8_t)(cell_face(0, dx, false) & cell_face(1, dy, false) & cell_face(2, dz, false))};
}
// The 13 backward cell neighbours (the other 13 are their mirror images).
__constant__ CellNb kCellNb[13] = {
    cell_nb(-1, -1, -1), cell_nb(-1, -1, 0), cell_nb(-1, -1, 1), cell_nb(-1, 0, -1), cell_nb(-1, 0, 0),
    cell_nb(-1, 0, 1),   cell_nb(-1, 1, -1), cell_nb(-1, 1, 0),  cell_nb(-1, 1, 1),  cell_nb(0, -1, -1),
    cell_nb(0, -1, 0),   cell_nb(0, -1, 1),  cell_nb(0, 0, -1)};

// Occupancy of a halo-framed block of cells: the tile's cells plus one cell on each x
// and y side and one layer below (cell coordinates -1 .. kC? along each axis).
constexpr int kHX = kCX + 2, kHY = kCY + 2, kHZ = kCZ + 1;
constexpr int kHalo = kHX * kHY * kHZ;        // 5780
__device__ __forceinline__ int halo_of(int cx, int cy, int cz) { return ((cz + 1) * kHY + (cy + 1)) * kHX + (cx + 1); }
__device__ __forceinline__ int cell_bit(int lx, int ly, int lz) { return ((lz & 1) << 2) | ((ly & 1) << 1) | (lx & 1); }

// Occupancy of the cell whose first voxel is (x, y, z) (volume coordinates; voxels outside
// the volume, past depth_valid handling or at index 0 count as background).
__device__ __forceinline__ uint32_t cell_occ(const Sub &S, const uint8_t *m, int64_t WH, int x, int y, int z) {
  uint32_t o = 0;
  if (x + 1 < 0 || x >= S.W || y + 1 < 0 || y >= S.H || z + 1 < 0 || z >= S.D) return 0;
  const bool pair = x >= 0 && x + 1 < S.W && (S.W % 2 == 0);
#pragma unroll
  for (int dz = 0; dz < 2; dz++)
#pragma unroll
    for (int dy = 0; dy < 2; dy++) {
      const int zz = z + dz, yy = y + dy;
      if (zz < 0 || zz >= S.D || yy < 0 || yy >= S.H) continue;
      const int64_t g = zz * WH + (int64_t)yy * S.W + x;
      uint32_t v;
      if (pair) {
        const uint16_t two = __ldg(reinterpret_cast<const uint16_t *>(m + g));
        v = ((two & 0xFFu) ? 1u : 0u) | ((two >> 8) ? 2u : 0u);
      } else {
        v = (x >= 0 && m[g]) ? 1u : 0u;
        if (x + 1 < S.W && m[g + 1]) v |= 2u;
      }
      if (g == 0) v &= ~1u;   // voxel 0 is background
      o |= v << (4 * dz + 2 * dy);
    }
  return o;
}

// Occupancy of the 8 cells whose first voxels are (x + 2k, y, z), k = 0..7, from one
// 16-byte load of each of the 4 voxel rows they cover (x 16-byte aligned, x + 15 < W;
// rows outside the volume read as background).
__device__ __forceinline__ void cell_occ8(const Sub &S, const uint8_t *m, int64_t WH, int x, int y, int z,
                                          uint32_t (&o)[8]) {
  uint4 r[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int zz = z + (q >> 1), yy = y + (q & 1);
    r[q] = (zz >= 0 && zz < S.D && yy >= 0 && yy < S.H)
               ? __ldg(reinterpret_cast<const uint4 *>(m + zz * WH + (int64_t)yy * S.W + x))
               : make_uint4(0u, 0u, 0u, 0u);
  }
#pragma unroll
  for (int k = 0; k < 8; k++) o[k] = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int sh = 4 * (q >> 1) + 2 * (q & 1);   // bit of the row's first voxel: 4 dz + 2 dy
    const uint32_t w[4] = {r[q].x, r[q].y, r[q].z, r[q].w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const uint32_t nz = __vcmpne4(w[j], 0u);   // 0xFF per foreground byte
      o[2 * j] |= ((nz & 1u) | ((nz >> 7) & 2u)) << sh;
      o[2 * j + 1] |= (((nz >> 16) & 1u) | ((nz >> 23) & 2u)) << sh;
    }
  }
}

// Drops links that other links of the tile already imply.  Every tile edge is linked by
// the later of its two cells, so with cell c linked to B (a backward neighbour) and B
// touching A (another backward neighbour of c), the edge B-A is linked too and c-A adds
// nothing.  Links kept unconditionally: k = 4 (dz -1), 10 (dy -1), 12 (dx -1).  Pruned:
//   via k = 4  (the cell below):  the other eight cells of the layer below, through the
//              in-plane edges of that layer;
//   via k = 10 (the cell behind): k = 9, 11 through that row's x edges (kept by rule) and
//              k = 1 through its own link k = 4 (kept);
//   via k = 12 (the cell left):   k = 9 through its link k = 10 and k = 3 through its
//              link k = 4 (both kept).
// Each pruned link rests on links that are kept or pruned only by the rules for
// in-layer edges, which rest on kept links: the implied connectivity is exact.
// The component minima are unchanged (they come from the final trees, not the links).
__device__ __forceinline__ bool touches(uint32_t a, uint32_t b, CellNb e) { return (a & e.self) && (b & e.other); }

__device__ __forceinline__ uint32_t prune_links(uint32_t todo, const uint32_t (&on)[13]) {
  if (todo & (1u << 4)) {
#pragma unroll
    for (int k = 0; k < 9; k++) {
      if (k == 4) continue;
      if (touches(on[4], on[k], cell_nb(0, k / 3 - 1, k % 3 - 1))) todo &= ~(1u << k);
    }
  }
  if (todo & (1u << 10)) {
    if (touches(on[10], on[9], cell_nb(0, 0, -1))) todo &= ~(1u << 9);
    if (touches(on[10], on[11], cell_nb(0, 0, 1))) todo &= ~(1u << 11);
    if (touches(on[10], on[1], cell_nb(-1, 0, 0))) todo &= ~(1u << 1);
  }
  if (todo & (1u << 12)) {
    if (touches(on[12], on[9], cell_nb(0, -1, 0))) todo &= ~(1u << 9);
    if (touches(on[12], on[3], cell_nb(-1, 0, 0))) todo &= ~(1u << 3);
  }
  return todo;
}

__global__ void __launch_bounds__(kCclThreads, 4) k_ccl_local(const Sub *subs, const uint8_t *mask, int32_t *labels,
                                                          int2 *edges, unsigned long long *edge_count) {
  __shared__ uint32_t par[kCells];
  __shared__ uint8_t occ[kHalo];
  __shared__ uint32_t minv[kCells];
  __shared__ int2 ebuf[kEdgeBuf];
  __shared__ uint32_t n_local_edges;
  __shared__ unsigned long long edge_base;
  const Sub S = subs[blockIdx.y];
  CclTile T;
  if (!ccl_tile(S, blockIdx.x, T)) return;
  const int t = threadIdx.x;
  const int64_t WH = (int64_t)S.W * S.H;
  const int64_t N = WH * S.D;
  const uint8_t *m = mask + S.vox;
  if (t == 0) n_local_edges = 0;
  // 1. occupancy of the tile's cells and of the halo (the layer below only when the tile
  //    does not start at slice 0); union-find nodes for the tile's cells.  Rows of 16-byte
  //    aligned tiles inside the volume are read 16 voxels (8 cells) per load; the halo's
  //    side columns, and every cell of other tiles, one cell at a time.
  const int ncz = (T.tz + 1) / 2;
  const bool rows16 = S.W % 16 == 0 && T.x0 + kTX <= S.W && (reinterpret_cast<uintptr_t>(m) & 15u) == 0;
  if (rows16) {
    constexpr int kSeg = kCX / 8;   // 8-cell segments per cell row
    for (int it = t; it < kHY * kHZ * kSeg; it += kCclThreads) {
      const int seg = it % kSeg, hy = (it / kSeg) % kHY, hz = it / (kSeg * kHY);
      const int cy = hy - 1, cz = hz - 1, cx0 = seg * 8;
      uint32_t o[8];
      if (cz < ncz && (cz >= 0 || T.z0 > 0)) {
        cell_occ8(S, m, WH, T.x0 + 2 * cx0, T.y0 + 2 * cy, T.z0 + 2 * cz, o);
        if (T.x0 == 0 && T.y0 + 2 * cy == 0 && T.z0 + 2 * cz == 0 && cx0 == 0) o[0] &= ~1u;   // voxel 0
        if (cz >= 0 && 2 * cz + 1 >= T.tz)
#pragma unroll
          for (int k = 0; k < 8; k++) o[k] &= 0x0Fu;
      } else {
#pragma unroll
        for (int k = 0; k < 8; k++) o[k] = 0;
      }
#pragma unroll
      for (int k = 0; k < 8; k++) occ[halo_of(cx0 + k, cy, cz)] = (uint8_t)o[k];
      if (cy >= 0 && cy < kCY && cz >= 0) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const int c = (cz * kCY + cy) * kCX + cx0 + k;
          par[c] = o[k] ? (uint32_t)c : kBg32;
          minv[c] = 0xFFFFFFFFu;
        }
      }
    }
  }
  for (int h = t; h < (rows16 ? kHY * kHZ * 2 : kHalo); h += kCclThreads) {
    int hx, hy, hz;
    if (rows16) {   // the side columns cx = -1 and cx = kCX
      hx = (h & 1) ? kHX - 1 : 0;
      hy = (h >> 1) % kHY;
      hz = (h >> 1) / kHY;
    } else {
      hx = h % kHX;
      hy = (h / kHX) % kHY;
      hz = h / (kHX * kHY);
    }
    const int cx = hx - 1, cy = hy - 1, cz = hz - 1;
    uint32_t o = 0;
    if (cz < ncz && (cz >= 0 || T.z0 > 0)) {
      o = cell_occ(S, m, WH, T.x0 + 2 * cx, T.y0 + 2 * cy, T.z0 + 2 * cz);
      if (cz >= 0 && 2 * cz + 1 >= T.tz) o &= 0x0Fu;   // a tile's last odd slice: no second layer
    }
    occ[(hz * kHY + hy) * kHX + hx] = (uint8_t)o;
    if (cx >= 0 && cx < kCX && cy >= 0 && cy < kCY && cz >= 0) {
      const int c = (cz * kCY + cy) * kCX + cx;
      par[c] = o ? (uint32_t)c : kBg32;
      minv[c] = 0xFFFFFFFFu;
    }
  }
  __syncthreads();
  // 2. unions between neighbouring cells of the tile.  The unrolled neighbour tests only
  //    collect a 13-bit list per cell, parked in minv (unused until step 3); the unions then
  //    run in warp-wide rounds over the lane's whole cell column, one link per lane and
  //    round, re-converged after each, so lanes whose finds and retries differ in length do
  //    not split the warp, and a lane with many links in one layer does not hold the
  //    others idle for that layer alone.  Union order does not change the components.
  const int cx = t % kCX, cy = t / kCX;
  uint32_t layers = 0;   // bit cz: the cell of layer cz has links
  for (int cz = 0; cz < ncz; cz++) {
    const int c = (cz * kCY + cy) * kCX + cx;
    const uint32_t oc = occ[halo_of(cx, cy, cz)];
    uint32_t todo = 0;
    if (oc) {
      uint32_t on[13];   // occupancy of the backward neighbours inside the tile (0 outside)
#pragma unroll
      for (int k = 0; k < 13; k++) {
        const CellNb nb = kCellNb[k];
        const int nx = cx + nb.dx, ny = cy + nb.dy, nz = cz + nb.dz;
        on[k] = (nx < 0 || nx >= kCX || ny < 0 || ny >= kCY || nz < 0) ? 0u : occ[halo_of(nx, ny, nz)];
        if ((oc & nb.self) && (on[k] & nb.other)) todo |= 1u << k;
      }
      todo = prune_links(todo, on);
    }
    minv[c] = todo;
    layers |= (todo ? 1u : 0u) << cz;
  }
  {
    uint32_t todo = 0;
    int c = 0;
    while (__any_sync(0xFFFFFFFFu, todo != 0 || layers != 0)) {
      if (!todo && layers) {
        const int cz = __ffs(layers) - 1;
        layers &= layers - 1;
        c = (cz * kCY + cy) * kCX + cx;
        todo = minv[c];
      }
      if (todo) {
        const int k = __ffs(todo) - 1;
        todo &= todo - 1;
        // backward cell offset k: (dz, dy, dx) as in kCellNb
        const int dz = k < 9 ? -1 : 0;
        const int dy = k < 9 ? k / 3 - 1 : (k < 12 ? -1 : 0);
        const int dx = k < 9 ? k % 3 - 1 : (k < 12 ? k - 10 : -1);
        const int cn = c + (dz * kCY + dy) * kCX + dx;
        if (par[cn] != par[c]) sunion(par, c, cn, 2 * kCells);
      }
      __syncwarp();
    }
  }
  for (int cz = 0; cz < ncz; cz++) minv[(cz * kCY + cy) * kCX + cx] = 0xFFFFFFFFu;
  __syncthreads();
  // 3. roots in place, then each component's minimum voxel (tile order = volume order)
  for (int cz = 0; cz < ncz; cz++) {
    const int c = (cz * kCY + cy) * kCX + cx;
    if (occ[halo_of(cx, cy, cz)]) par[c] = sroot(par, c);
  }
  __syncthreads();
  for (int cz = 0; cz < ncz; cz++) {
    const int c = (cz * kCY + cy) * kCX + cx;
    const uint32_t oc = occ[halo_of(cx, cy, cz)];
    if (!oc) continue;
    const int b = __ffs(oc) - 1;   // first voxel of the cell in linear order
    const uint32_t v = ((2 * cz + (b >> 2)) * kTY + 2 * cy + ((b >> 1) & 1)) * kTX + 2 * cx + (b & 1);
    atomicMin(&minv[par[c]], v);
  }
  // 4a. plain cross-tile edges, cell to cell: a face cell and its backward neighbour cell
  //     outside the tile are connected when their facing voxels are foreground; the edge
  //     joins the first foreground voxel of each
  auto first_voxel = [&](int ccx, int ccy, int ccz, uint32_t o) -> int64_t {
    const int b = __ffs(o) - 1;
    return (int64_t)(T.z0 + 2 * ccz + (b >> 2)) * WH + (int64_t)(T.y0 + 2 * ccy + ((b >> 1) & 1)) * S.W + T.x0 +
           2 * ccx + (b & 1);
  };
  auto emit = [&](int64_t a, int64_t b) {
    const uint32_t i = atomicAdd(&n_local_edges, 1u);
    if (i < (uint32_t)kEdgeBuf) {
      ebuf[i] = make_int2((int32_t)a, (int32_t)b);
    } else {
      const unsigned long long j = atomicAdd(&edge_count[blockIdx.y], 1ull);
      if ((int64_t)j < S.edge_cap) edges[S.edge + j] = make_int2((int32_t)a, (int32_t)b);
    }
  };
  {
    constexpr int kFacePerLayer = 2 * kCX + 2 * (kCY - 2);   // rows cy = 0, kCY-1 and columns cx = 0, kCX-1
    const bool zface = T.z0 > 0;
    const int nf = zface ? ncz * kFacePerLayer + kCX * kCY : ncz * kFacePerLayer;
    for (int f = t; f < nf; f += kCclThreads) {
      int fx, fy, fz;
      if (f < ncz * kFacePerLayer) {
        fz = f / kFacePerLayer;
        const int j = f % kFacePerLayer;
        if (j < kCX) { fx = j; fy = 0; }
        else if (j < 2 * kCX) { fx = j - kCX; fy = kCY - 1; }
        else if (j < 2 * kCX + kCY - 2) { fx = 0; fy = j - 2 * kCX + 1; }
        else { fx = kCX - 1; fy = j - 2 * kCX - (kCY - 2) + 1; }
      } else {   // the bottom layer of a tile above slice 0, interior cells (faces done above)
        const int j = f - ncz * kFacePerLayer;
        fx = j % kCX; fy = j / kCX; fz = 0;
        if (fx == 0 || fx == kCX - 1 || fy == 0 || fy == kCY - 1) continue;
      }
      const uint32_t oc = occ[halo_of(fx, fy, fz)];
      if (!oc) continue;
      uint32_t todo = 0;
#pragma unroll
      for (int k = 0; k < 13; k++) {
        const CellNb nb = kCellNb[k];
        const int nx = fx + nb.dx, ny = fy + nb.dy, nz = fz + nb.dz;
        if (nx >= 0 && nx < kCX && ny >= 0 && ny < kCY && nz >= 0) continue;   // inside the tile
        if (nz < 0 && !zface) continue;
        if ((oc & nb.self) && (occ[halo_of(nx, ny, nz)] & nb.other)) todo |= 1u << k;
      }
      if (!todo) continue;
      const int64_t a = first_voxel(fx, fy, fz, oc);
      while (todo) {
        const int k = __ffs(todo) - 1;
        todo &= todo - 1;
        const int dz = k < 9 ? -1 : 0;
        const int dy = k < 9 ? k / 3 - 1 : (k < 12 ? -1 : 0);
        const int dx = k < 9 ? k % 3 - 1 : (k < 12 ? k - 10 : -1);
        const int nx = fx + dx, ny = fy + dy, nz = fz + dz;
        emit(a, first_voxel(nx, ny, nz, occ[halo_of(nx, ny, nz)]));
      }
    }
  }
  // 4b. the reference's wrap-around edges: backward linear offsets of a voxel in the first
  //     or last column or row that leave the row or slice (only border tiles hold such voxels)
  if (T.x0 == 0 || T.x0 + kTX >= S.W || T.y0 == 0 || T.y0 + kTY >= S.H) {
    const int lastx = min(kTX - 1, S.W - 1 - T.x0), lasty = min(kTY - 1, S.H - 1 - T.y0);
    for (int v = t; v < kTX * kTY * T.tz; v += kCclThreads) {
      const int lx = v % kTX, ly = (v / kTX) % kTY, lz = v / (kTX * kTY);
      if (lx > lastx || ly > lasty) continue;
      const int x = T.x0 + lx, y = T.y0 + ly, z = T.z0 + lz;
      if (x != 0 && x != S.W - 1 && y != 0 && y != S.H - 1) continue;
      if (!((occ[halo_of(lx >> 1, ly >> 1, lz >> 1)] >> cell_bit(lx, ly, lz)) & 1u)) continue;
      const int64_t g = z * WH + (int64_t)y * S.W + x;
      for (int o = 0; o < 13; o++) {
        int dz, dy, dx;
        back_offset(o, dz, dy, dx);
        if (x + dx >= 0 && x + dx < S.W && y + dy >= 0 && y + dy < S.H) continue;   // a plain step
        const int64_t gn = g + dz * WH + dy * (int64_t)S.W + dx;
        if (gn >= 1 && gn < N && m[gn]) emit(g, gn);
      }
    }
  }
  __syncthreads();
  // 5. staged edges to their global slots
  if (t == 0) {
    const uint32_t ne = min(n_local_edges, (uint32_t)kEdgeBuf);
    edge_base = ne ? atomicAdd(&edge_count[blockIdx.y], (unsigned long long)ne) : 0ull;
  }
  __syncthreads();
  {
    const uint32_t ne = min(n_local_edges, (uint32_t)kEdgeBuf);
    for (uint32_t i = t; i < ne; i += kCclThreads) {
      const unsigned long long j = edge_base + i;
      if ((int64_t)j < S.edge_cap) edges[S.edge + j] = ebuf[i];
    }
  }
  // 6. labels: the component's minimum voxel as a global index, background -> 0.  First
  //    every occupied cell's label, once per cell, into par (whose roots are no longer
  //    needed), then whole rows of voxels from their cells' labels (vector stores).
  for (int cz = 0; cz < ncz; cz++) {
    const int c = (cz * kCY + cy) * kCX + cx;
    if (!occ[halo_of(cx, cy, cz)]) continue;
    const uint32_t r = minv[par[c]];
    par[c] = (uint32_t)((T.z0 + (int)(r / (kTX * kTY))) * WH + (int64_t)(T.y0 + (int)((r / kTX) % kTY)) * S.W +
                        T.x0 + (int)(r % kTX));
  }
  __syncthreads();
  const int lx0 = (t % (kTX / 4)) * 4, ly = t / (kTX / 4);
  const int x = T.x0 + lx0, y = T.y0 + ly;
  if (y >= S.H) return;
  const bool vec = x + 3 < S.W && (S.W % 4 == 0);
  int32_t *L = labels + S.vox;
  const int c0x = lx0 >> 1;   // the quad's voxels lie in cells c0x (first two) and c0x + 1
  for (int lz = 0; lz < T.tz; lz++) {
    const int64_t g = (T.z0 + lz) * WH + (int64_t)y * S.W + x;
    const int b = ((lz & 1) << 2) | ((ly & 1) << 1);   // bit of the even-x voxel in its cell
    const uint32_t o0 = occ[halo_of(c0x, ly >> 1, lz >> 1)] >> b, o1 = occ[halo_of(c0x + 1, ly >> 1, lz >> 1)] >> b;
    const int cb = ((lz >> 1) * kCY + (ly >> 1)) * kCX + c0x;
    const int32_t l0 = (o0 & 3u) ? (int32_t)par[cb] : 0, l1 = (o1 & 3u) ? (int32_t)par[cb + 1] : 0;
    int32_t out[4] = {(o0 & 1u) ? l0 : 0, (o0 & 2u) ? l0 : 0, (o1 & 1u) ? l1 : 0, (o1 & 2u) ? l1 : 0};
    if (vec) {
      *reinterpret_cast<int4 *>(L + g) = make_int4(out[0], out[1], out[2], out[3]);
    } else {
#pragma unroll
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
    uf_union(L, ab.x, ab.y, S.walk_limit > 0 ? S.walk_limit : n, status);
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
        if (gn >= 1 && m[gn]) uf_union(L, (int32_t)g, (int32_t)gn, S.walk_limit > 0 ? S.walk_limit : n, status);
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
    // level by level over the 16 voxels: their labels, then the labels' parents, so the
    // loads of a level are in flight together; deeper walks (labels merged across tiles
    // more than once) continue one by one
    int32_t l[16], p[16];
#pragma unroll
    for (int k = 0; k < 16; k++) l[k] = (mk[k] && i0 + k != 0) ? __ldcg(L + i0 + k) : -1;
#pragma unroll
    for (int k = 0; k < 16; k++) p[k] = l[k] >= 0 ? __ldcg(L + l[k]) : -1;
#pragma unroll
    for (int k = 0; k < 16; k++) {
      if (l[k] < 0) continue;
      const int32_t r = p[k] == l[k] ? l[k] : uf_root(L, p[k], S.walk_limit > 0 ? S.walk_limit : n, status);
      if (r != l[k]) L[i0 + k] = r;
      if (r == (int32_t)(i0 + k)) bits |= 1u << k;
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

// The same pass over the fused sweep's foreground list instead of the whole volume (the list
// holds every foreground voxel but voxel 0): root bits and block counts start at zero and
// each root sets its own bit and counts itself.  fg_root holds each entry's voxel index
// (written by the sweep beside the 32-byte entry, so that this pass reads 4 bytes per
// entry) and is overwritten with the entry's root.  A substack whose list overflowed is
// skipped; its batch is redone with the separate passes.
constexpr int kFlatFgPerThread = 16;

__global__ void __launch_bounds__(256) k_ccl_flatten_fg(const Sub *subs, const unsigned long long *fg_count,
                                                       int32_t *labels,
                                                       uint32_t *root_bits, uint32_t *blk_counts, int32_t *fg_root,
                                                       int *status) {
  const Sub S = subs[blockIdx.y];
  const int64_t cnt = (int64_t)fg_count[blockIdx.y * kFgCountStride];
  if (cnt > S.fg_cap) return;
  const int64_t n = (int64_t)S.W * S.H * S.D;
  int32_t *L = labels + S.vox;
  // a warp takes 32 * kFlatFgPerThread consecutive entries, lane l every 32nd from l, so each
  // load and store of the warp covers 32 consecutive entries
  const int lane = threadIdx.x & 31;
  const int64_t span = 32 * kFlatFgPerThread;
  const int64_t stride = ((int64_t)gridDim.x * blockDim.x >> 5) * span;
  for (int64_t w0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * span; w0 < cnt; w0 += stride) {
    const int64_t e0 = w0 + lane;   // entries e0 + 32 k
    // level by level: the entries' voxels, their labels, the labels' parents
    int32_t idx[kFlatFgPerThread], l[kFlatFgPerThread], p[kFlatFgPerThread];
#pragma unroll
    for (int k = 0; k < kFlatFgPerThread; k++) idx[k] = e0 + 32 * k < cnt ? fg_root[S.fg + e0 + 32 * k] : -1;
#pragma unroll
    for (int k = 0; k < kFlatFgPerThread; k++) l[k] = idx[k] >= 0 ? __ldcg(L + idx[k]) : -1;
#pragma unroll
    for (int k = 0; k < kFlatFgPerThread; k++) p[k] = l[k] >= 0 ? __ldcg(L + l[k]) : -1;
#pragma unroll
    for (int k = 0; k < kFlatFgPerThread; k++) {
      if (l[k] < 0) continue;
      const int32_t r = p[k] == l[k] ? l[k] : uf_root(L, p[k], S.walk_limit > 0 ? S.walk_limit : n, status);
      if (r != l[k]) L[idx[k]] = r;
      fg_root[S.fg + e0 + 32 * k] = r;   // the entry's root, read by the region accumulation
      if (r == idx[k]) {
        const int64_t b = idx[k] / kScanBlock;
        const int o = (int)(idx[k] % kScanBlock);
        atomicOr(root_bits + (S.blk + b) * (kScanBlock / 32) + o / 32, 1u << (o % 32));
        atomicAdd(blk_counts + S.blk + b, 1u);
      }
    }
  }
}

// ------------------------------------------------------------------ launchers
void launch_ccl(const Sub *d_subs, int nsub, int max_w, int max_h, int max_d, int64_t max_n, const uint8_t *mask,
                int32_t *labels, int2 *edges, unsigned long long *edge_count, uint32_t *root_bits,
                uint32_t *blk_counts, int *d_status, int num_sms, cudaStream_t s, const FgEntry *fg,
                const unsigned long long *fg_count, int64_t max_fg, int64_t nblk, int32_t *fg_root) {
  const int64_t tiles = (int64_t)ceil_div(max_w, kTX) * ceil_div(max_h, kTY) * ceil_div(max_d, kTZ);
  zero_async(edge_count, nsub * sizeof(unsigned long long), s);
  KLAUNCH("k_ccl_local", s, (k_ccl_local<<<dim3((unsigned)tiles, nsub), kCclThreads, 0, s>>>(
                                d_subs, mask, labels, edges, edge_count)));
  const unsigned eb = (unsigned)max(1, (8 * num_sms + nsub - 1) / nsub);
  KLAUNCH("k_ccl_edges", s, (k_ccl_edges<<<dim3(eb, nsub), 256, 0, s>>>(d_subs, edges, edge_count, labels,
                                                                        d_status)));
  KLAUNCH("k_ccl_cross_direct", s, (k_ccl_cross_direct<<<dim3((unsigned)tiles, nsub), kCclThreads, 0, s>>>(
                                       d_subs, mask, edge_count, labels, d_status)));
  if (fg) {
    zero_async(root_bits, (size_t)nsub * nblk * (kScanBlock / 32) * sizeof(uint32_t), s);
    zero_async(blk_counts, (size_t)nsub * nblk * sizeof(uint32_t), s);
    const int64_t want = std::min((int64_t)ceil_div(max_fg, 256 * kFlatFgPerThread),
                                  (int64_t)(8 * num_sms / (nsub > 0 ? nsub : 1) + 1));
    KLAUNCH("k_ccl_flatten", s, (k_ccl_flatten_fg<<<dim3((unsigned)std::max<int64_t>(want, 1), nsub), 256, 0, s>>>(
                                    d_subs, fg_count, labels, root_bits, blk_counts, fg_root, d_status)));
  } else {
    KLAUNCH("k_ccl_flatten", s, (k_ccl_flatten<false><<<dim3(ceil_div(max_n, kScanBlock), nsub), 256, 0, s>>>(
                                    d_subs, const_cast<uint8_t *>(mask), labels, root_bits, blk_counts, d_status)));
  }
}

void launch_roots_from_labels(const Sub *d_subs, int nsub, int64_t max_n, const int32_t *labels, uint8_t *mask,
                              uint32_t *root_bits, uint32_t *blk_counts, cudaStream_t s) {
  KLAUNCH("k_roots_from_labels", s, (k_ccl_flatten<true><<<dim3(ceil_div(max_n, kScanBlock), nsub), 256, 0, s>>>(
                                        d_subs, mask, const_cast<int32_t *>(labels), root_bits, blk_counts,
                                        nullptr)));
}

}  // namespace hdog
