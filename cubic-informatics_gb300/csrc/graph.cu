// graph.cu -- device steps of the batched graph form (hdog_graph_*): after each batch of a
// captured run, the records of its substacks are placed in one device array of the whole
// run, and a redo flag is raised when a batch needs the host's fallback.
//
// The reference has no batched form: HDoG3D_main runs its substacks one at a time and
// appends each substack's records to the stack's file (src/3D/HDoG3D_main.cpp:294-315,
// src/3D/utils.h:204-250).  The placement below keeps that order: every substack's records
// land contiguously, in label order, and the host reads them back substack by substack in
// the caller's stack order.
#include "kernels.cuh"

namespace hdog {

// One thread: each batch substack's slot in the run's record array, after the running
// total.  A batch whose foreground list overflowed, whose status word is set, or whose
// records would pass the array's end raises *redo (the host then reruns the call without
// the graph); the copy below skips what does not fit.
__global__ void k_graph_place(int nsub, GraphIds ids, const int64_t *num_records, const unsigned long long *fg_count,
                              int64_t fg_cap, int fused, const int *status, int64_t *total, GraphSlot *table, int *redo,
                              int64_t out_cap) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int64_t t = *total;
  int bad = *status != 0;
  for (int s = 0; s < nsub; s++) {
    const int64_t k = num_records[s];
    table[ids.id[s]].off = t;
    table[ids.id[s]].count = k;
    t += k;
    if (fused && fg_count[(int64_t)s * kFgCountStride] > (unsigned long long)fg_cap) bad = 1;
  }
  if (t > out_cap) bad = 1;
  if (bad) *redo = 1;
  *total = t;
}

// Copies substack blockIdx.y's records (28-byte structs, as 32-bit words) to its slot.
__global__ void k_graph_copy(GraphIds ids, const hdog_record *records, int64_t reg_cap, const GraphSlot *table,
                             hdog_record *out, int64_t out_cap) {
  const int s = blockIdx.y;
  const GraphSlot slot = table[ids.id[s]];
  int64_t n = slot.count;
  if (slot.off + n > out_cap) n = slot.off < out_cap ? out_cap - slot.off : 0;
  constexpr int kWords = (int)(sizeof(hdog_record) / 4);
  const uint32_t *src = reinterpret_cast<const uint32_t *>(records + (int64_t)s * reg_cap);
  uint32_t *dst = reinterpret_cast<uint32_t *>(out + slot.off);
  const int64_t words = n * kWords;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

void launch_graph_place(int nsub, const GraphIds &ids, const int64_t *num_records, const unsigned long long *fg_count,
                        int64_t fg_cap, bool fused, const int *status, int64_t *total, GraphSlot *table, int *redo,
                        int64_t out_cap, cudaStream_t s) {
  KLAUNCH("k_graph_place", s, (k_graph_place<<<1, 32, 0, s>>>(nsub, ids, num_records, fg_count, fg_cap, fused ? 1 : 0,
                                                              status, total, table, redo, out_cap)));
}

void launch_graph_copy(int nsub, const GraphIds &ids, const hdog_record *records, int64_t reg_cap,
                       const GraphSlot *table, hdog_record *out, int64_t out_cap, cudaStream_t s) {
  KLAUNCH("k_graph_copy", s, (k_graph_copy<<<dim3(96, nsub), 256, 0, s>>>(ids, records, reg_cap, table, out, out_cap)));
}

}  // namespace hdog
