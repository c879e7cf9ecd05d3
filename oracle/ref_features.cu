// ref_features.cu -- TEST INFRASTRUCTURE ONLY (the checker, never linked into libhdog).
//
// The region reductions of the reference's HDoG3D_main, restated call for call with the
// same CUB device algorithms on the same inputs, so that records built from the reference's
// own stage kernels (oracle/ref_cubin.py) get their float sums by the reference's method:
//   HessianFeatures           src/3D/RegionalFeatures.cu:295-329   per Hessian plane:
//                             DeviceRadixSort::SortPairs(label -> value), DeviceReduce::ReduceByKey(a + b)
//   MaxNormalized             src/3D/RegionalFeatures.cu:65-87     SortPairs(label -> norm), ReduceByKey((b > a) ? b : a)
//   SumNormalized             src/3D/RegionalFeatures.cu:114-137   SortPairs(label -> norm), ReduceByKey(a + b)
//   RegionalSizeAndCentroid   src/3D/RegionalFeatures.cu:157-255   per axis: coordinate plane as float,
//                             SortPairs, ReduceByKey(a + b); DeviceRunLengthEncode::Encode of the sorted
//                             labels into unsigned short counts; each coordinate sum /= its count
// The order of the calls and their arguments follow HDoG3D_main.cpp:178-210.  CUB itself is the
// toolkit's (the CCCL of CUDA 13.0 where this is built; the reference's Docker image pins CUDA
// 11.6), so the association inside ReduceByKey is this CUB's: float sums are reproduced to the
// library's order, not to the bit of a CUDA 11.6 build.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cub/cub.cuh>

namespace {

struct MaxOf {
  __device__ __forceinline__ float operator()(const float &a, const float &b) const { return (b > a) ? b : a; }
};
struct SumOf {
  __device__ __forceinline__ float operator()(const float &a, const float &b) const { return a + b; }
};

__global__ void k_coordinate(float *grid, int axis, int w, int h, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = i % w, y = (i / w) % h, z = i / ((int64_t)w * h);
    grid[i] = (float)(axis == 0 ? x : (axis == 1 ? y : z));
  }
}

__global__ void k_divide(float *v, const unsigned short *count, int k) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) v[i] /= count[i];
}

struct Scratch {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t need(size_t b) {
    if (b <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  ~Scratch() {
    if (p) cudaFree(p);
  }
};

#define CK(x)                              \
  do {                                     \
    cudaError_t e__ = (x);                 \
    if (e__ != cudaSuccess) return (int)e__; \
  } while (0)

#define CKI(x)          \
  do {                  \
    int r__ = (x);      \
    if (r__) return r__; \
  } while (0)

template <class Op>
int sort_reduce(Scratch &tmp, const int *labels, const float *values, int *labels_tmp, float *values_tmp,
                int *labels_reg, float *out_reg, int *num_regions, Op op, int n) {
  size_t b = 0;
  CK(cub::DeviceRadixSort::SortPairs(nullptr, b, labels, labels_tmp, values, values_tmp, n));
  CK(tmp.need(b));
  CK(cub::DeviceRadixSort::SortPairs(tmp.p, b, labels, labels_tmp, values, values_tmp, n));
  b = 0;
  CK(cub::DeviceReduce::ReduceByKey(nullptr, b, labels_tmp, labels_reg, values_tmp, out_reg, num_regions, op, n));
  CK(tmp.need(b));
  CK(cub::DeviceReduce::ReduceByKey(tmp.p, b, labels_tmp, labels_reg, values_tmp, out_reg, num_regions, op, n));
  return 0;
}

}  // namespace

// All arrays are device memory of n = w*h*d elements (region outputs hold num_regions < n of
// them, at pitch n where there are several rows): labels (CCL output), hessian (six planes
// xx, xy, xz, yy, yz, zz), norm; scratch labels_tmp, values_tmp, labels_reg, grid.  Outputs:
// hess_reg [6][n], intensity_reg [n] (max, or sum when is_ave), size_reg [n] (unsigned short),
// centroid_reg [3][n], *num_regions.  Returns a cudaError_t code.
extern "C" int ref_regional_features(const int *labels, const float *hessian, const float *norm, int w, int h, int d,
                                     int is_ave, int *labels_tmp, float *values_tmp, int *labels_reg, float *grid,
                                     float *hess_reg, float *intensity_reg, unsigned short *size_reg,
                                     float *centroid_reg, int *num_regions) {
  const int n = w * h * d;   // int, as the reference's image_size
  Scratch tmp;
  for (int i = 0; i < 6; i++)
    CKI(sort_reduce(tmp, labels, hessian + (size_t)n * i, labels_tmp, values_tmp, labels_reg, hess_reg + (size_t)n * i,
                   num_regions, SumOf(), n));
  int h_num = 0;
  CK(cudaMemcpy(&h_num, num_regions, sizeof(int), cudaMemcpyDeviceToHost));
  if (is_ave)
    CKI(sort_reduce(tmp, labels, norm, labels_tmp, values_tmp, labels_reg, intensity_reg, num_regions, SumOf(), n));
  else
    CKI(sort_reduce(tmp, labels, norm, labels_tmp, values_tmp, labels_reg, intensity_reg, num_regions, MaxOf(), n));
  for (int axis = 0; axis < 3; axis++) {
    k_coordinate<<<1024, 256>>>(grid, axis, w, h, (int64_t)n);
    CK(cudaGetLastError());
    CKI(sort_reduce(tmp, labels, grid, labels_tmp, values_tmp, labels_reg, centroid_reg + (size_t)n * axis, num_regions,
                   SumOf(), n));
  }
  size_t b = 0;
  CK(cub::DeviceRunLengthEncode::Encode(nullptr, b, labels_tmp, labels_reg, size_reg, num_regions, n));
  CK(tmp.need(b));
  CK(cub::DeviceRunLengthEncode::Encode(tmp.p, b, labels_tmp, labels_reg, size_reg, num_regions, n));
  for (int axis = 0; axis < 3; axis++) {
    k_divide<<<256, 256>>>(centroid_reg + (size_t)n * axis, size_reg, h_num);
    CK(cudaGetLastError());
  }
  CK(cudaDeviceSynchronize());
  return 0;
}
