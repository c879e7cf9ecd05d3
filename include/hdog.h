/*
 * hdog.h -- C ABI of the GB300 HDoG cell-candidate detection library (libhdog.so).
 *
 * Drop-in for the HDoG hot path of CUBIC-informatics (src/3D).  Plain C types only:
 * device buffers are `void *`/typed pointers, CUDA streams are passed as `void *`
 * (a cudaStream_t; NULL = the legacy default stream).  Every function returns an
 * HDOG_* status; none calls exit() (the reference exits through helper_cuda.h:595-612
 * and utils.h:97-100).  hdog_last_error() gives the message of the last failure on the
 * calling thread.
 *
 * Reference interfaces replaced (file:line within the reference project):
 *   hdog_run_param_file     HDoG3D_main executable           src/3D/HDoG3D_main.cpp:260-319
 *   hdog_params_load_json   loadParamFile                    src/3D/utils.h:95-157
 *   hdog_gaussian_taps      calcGaussianWeight               src/3D/DoG3DFilter.cu:372-392
 *   hdog_depth_margin       initGaussian3DKernel + margin    src/3D/DoG3DFilter.cu:394-415,
 *                                                            src/3D/HDoG3D_main.cpp:280-284
 *   hdog_normalize          Normalize3DFilter                src/3D/NormalizeFilter.cu:603-654
 *   hdog_dog                DoG3DFilter                      src/3D/DoG3DFilter.cu:431-437
 *   hdog_hessian_pd         HessianPositiveDefiniteWithElement
 *                                                            src/3D/Hessian3DFilter_element.cu:355-388
 *   hdog_ccl                CCL                              src/3D/CCL3D.cu:81-117
 *   hdog_regional_features  HessianFeatures + Eigenvalues + MaxNormalized / SumNormalized +
 *                           RegionalSizeAndCentroid          src/3D/RegionalFeatures.cu:65-87,
 *                                                            114-137,214-255,295-329;
 *                                                            src/3D/Eigenvalues.cu:99-112
 *   hdog_erosion            Erosion3DFilter                  src/3D/Erosion3DFilter.cu:260-268
 *   hdog_run_substack       processSubstack + saveFeatureVector
 *                                                            src/3D/HDoG3D_main.cpp:134-257,
 *                                                            src/3D/utils.h:204-250
 *   hdog_run_stack          the substack loop of main        src/3D/HDoG3D_main.cpp:294-315
 *   hdog_run_stacks         main's loop over the stacks of a parameter file
 *                                                            src/3D/HDoG3D_main.cpp:287-316
 *   hdog_records_to_global  HDoGResultStack                  script/HalfBrainCells.py:44-56
 *   hdog_scale_merge        process_stack (scale merge)      script/MergeBrain.py:546-570
 *   hdog_classifier_features get_X_3d                        script/HDoG_classifier.py:158-176
 */
#ifndef HDOG_H
#define HDOG_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HDOG_ABI_VERSION 5

enum {
  HDOG_OK = 0,
  HDOG_ERR_ARG = 1,       /* null pointer, negative or inconsistent size */
  HDOG_ERR_SHAPE = 2,     /* geometry or radius outside what the kernels support */
  HDOG_ERR_CUDA = 3,      /* CUDA runtime error (message has the detail) */
  HDOG_ERR_IO = 4,        /* file could not be opened, read or written */
  HDOG_ERR_PARAM = 5,     /* parameter file malformed or missing a required key */
  HDOG_ERR_CAPACITY = 6,  /* caller's output buffer (or region capacity) too small */
  HDOG_ERR_TIMEOUT = 7,   /* a bounded device loop hit its iteration limit */
  HDOG_ERR_NOMEM = 8
};

/* HDoG parameters, the keys HDoG3D_main reads (src/3D/utils.h:48-93). */
typedef struct hdog_params {
  int width, height;            /* input_image_info.width / height */
  int depth;                    /* HDoG_param.depth: slices per substack */
  int left_margin, right_margin, top_margin, bottom_margin;
  int extra_depth_margin;       /* HDoG_param.extra_depth_margin */
  int radius_norm_xy, radius_norm_z;   /* HDoG_param.radius_norm.{xy_large,z_large} */
  int min_intensity;            /* HDoG_param.min_intensity (unsigned short) */
  float gamma_n;                /* HDoG_param.gamma_n */
  float sigma_xy_small, sigma_z_small, sigma_xy_large, sigma_z_large;  /* sigma_dog */
  int min_size;                 /* HDoG_param.min_size (unsigned short) */
  int is_ave_mode;              /* top-level is_ave_mode: intensity = sum instead of max */
  int erosion_radius_xy, erosion_radius_z;  /* opt-in regional erosion of the input before
                                               normalization; 0,0 = off, as the reference */
  int dev_id;                   /* devID */
} hdog_params;

/* 28-byte candidate record == FeatureVector (src/3D/utils.h:188-197) == dt_local
   (script/HalfBrainCells.py:11-15). */
typedef struct hdog_record {
  float centroid_x, centroid_y, centroid_z;
  float structureness, blobness, intensity;
  uint16_t size, padding;
} hdog_record;

/* Per-region results of hdog_regional_features: DEVICE arrays owned by the context, valid
   until the next call on it.  Region 0 is the background; regions are ordered by label,
   i.e. by the minimum linear voxel index of the component. */
typedef struct hdog_regions {
  int64_t num_regions;          /* background included */
  const int32_t *label;         /* [num_regions] */
  const uint32_t *count;        /* [num_regions] exact voxel count (records keep count & 0xFFFF) */
  const float *intensity;       /* [num_regions] max (or sum, is_ave_mode) of normalized intensity */
  const float *centroid;        /* [3][pitch], first num_regions of each row: x, y, z (sum / (float)(uint16)count) */
  const float *hessian;         /* [6][pitch]: sums of xx, xy, xz, yy, yz, zz */
  const float *eigen;           /* [2][pitch]: structureness, blobness */
  int64_t pitch;                /* elements between the rows of centroid, hessian and eigen */
} hdog_regions;

typedef struct hdog_ctx hdog_ctx;

/* ---- errors, version ---- */
const char *hdog_last_error(void);
int hdog_abi_version(void);

/* ---- parameters ---- */
/* Fills *p from an HDoG parameter JSON file (loadParamFile semantics; '#' keys ignored). */
int hdog_params_load_json(const char *path, hdog_params *p);
/* Gaussian taps of calcGaussianWeight: taps[80], *radius = (int)(2*sigma + 0.5). */
int hdog_gaussian_taps(float sigma, float *taps80, int *radius);
/* depth_margin = radius of the large-z Gaussian + extra_depth_margin. */
int hdog_depth_margin(const hdog_params *p, int *margin);

/* ---- context: device scratch for up to max_substacks substacks of width x height x depth ---- */
int hdog_ctx_create(const hdog_params *p, int max_substacks, hdog_ctx **out);
int hdog_ctx_destroy(hdog_ctx *ctx);
/* Device scratch bytes hdog_ctx_create allocates for these parameters. */
int hdog_ctx_bytes(const hdog_params *p, int max_substacks, size_t *bytes);

/* ---- stages (device pointers, one substack of width x height x depth, on `stream`) ---- */
int hdog_normalize(hdog_ctx *ctx, const uint16_t *d_img, float *d_norm, void *stream);
/* hdog_normalize plus the two box means it divides by: d_ero_l = box mean of the min,
   d_dil_l = box mean of the max (the d_erosion_l / d_dilation_l of Normalize3DFilter,
   src/3D/NormalizeFilter.cu:603-654, dumped by test/Normalize_test.cpp:95-118).  With a
   normalization radius of 0 (the copy path, which computes no box means) both are zero. */
int hdog_normalize_parts(hdog_ctx *ctx, const uint16_t *d_img, float *d_norm, float *d_ero_l, float *d_dil_l,
                         void *stream);
/* Synchronizes `stream`: the radius-specialised sweep's bounded waits report a timeout
   (HDOG_ERR_TIMEOUT) through the call's return value. */
int hdog_dog(hdog_ctx *ctx, const float *d_norm, float *d_dog, void *stream);
/* d_hessian may be NULL; when given it receives the six planes xx,xy,xz,yy,yz,zz (pitch N). */
int hdog_hessian_pd(hdog_ctx *ctx, const float *d_dog, uint8_t *d_mask, float *d_hessian,
                    void *stream);
int hdog_ccl(hdog_ctx *ctx, const uint8_t *d_mask, int32_t *d_labels, void *stream);
/* Synchronizes `stream` to read the region count. */
int hdog_regional_features(hdog_ctx *ctx, const int32_t *d_labels, const float *d_norm,
                           const float *d_dog, hdog_regions *out, void *stream);
/* Regional erosion: min over a (2rxy+1)^2 (2rz+1) box with a zero border, x -> y -> z. */
int hdog_erosion(hdog_ctx *ctx, const uint16_t *d_src, uint16_t *d_dst, int radius_xy,
                 int radius_z, void *stream);

/* ---- whole chain ---- */
/* One substack: img holds depth_valid slices (host memory, or device memory when
   img_on_device != 0); slices depth_valid..depth-1 are taken as zero.  Records of
   regions that pass the margin/size/intensity filter go to out (host), at most cap of
   them; *n_records receives the number kept (HDOG_ERR_CAPACITY when it exceeds cap). */
int hdog_run_substack(hdog_ctx *ctx, const uint16_t *img, int img_on_device, int depth_valid,
                      int z0, hdog_record *out, int64_t cap, int64_t *n_records, void *stream);
/* One stack of `length` slices: the overlapping substack schedule of HDoG3D_main
   (z0 = 0, D-2m, ... while z0 < length - m), the substacks run as one batch when the
   context has room, records appended in substack order.  A host stack is copied in chunks
   that overlap the work (page-locked memory copies fastest); an out array in page-locked
   memory receives the records straight from the device. */
int hdog_run_stack(hdog_ctx *ctx, const uint16_t *stack, int stack_on_device, int length,
                   hdog_record *out, int64_t cap, int64_t *n_records, void *stream);
/* Many stacks of the context's width and height in one call: the substacks of all stacks
   (each stack in its own HDoG3D_main schedule) are packed into batches of as many as the
   context holds, across stack boundaries, so uneven stack lengths leave no partial batches
   but the last.  Records come out stack by stack, each stack's in substack order, exactly as
   hdog_run_stack gives them; stack_counts[i] (may be NULL) receives stack i's count.  Host
   stacks are copied to device memory the call allocates and frees. */
typedef struct hdog_stack_in {
  const uint16_t *data;   /* length slices of width * height uint16, x fastest */
  int on_device;          /* 1: device memory, 0: host memory */
  int length;             /* slices */
} hdog_stack_in;
int hdog_run_stacks(hdog_ctx *ctx, const hdog_stack_in *stacks, int n_stacks, hdog_record *out, int64_t cap,
                    int64_t *n_records, int64_t *stack_counts, void *stream);
/* The records of the context's last hdog_run_substack / hdog_run_stack / hdog_run_stacks call, kept by the
   context (also after that call returned HDOG_ERR_CAPACITY): a caller whose buffer was
   too small sizes a new one from *n_records and fetches them here instead of running
   the chain again.  No counterpart in the reference (HDoG3D_main writes records to a
   file as it goes). */
int hdog_last_records(hdog_ctx *ctx, hdog_record *out, int64_t cap, int64_t *n_records);
/* The HDoG3D_main executable as a call: reads the parameter file, processes every stack,
   writes each dst_path (removed first, then appended per substack). */
int hdog_run_param_file(const char *param_path, int verbose);

/* ---- the batched graph form ----
   Many stacks of uneven depth and frame shape in one captured CUDA graph.  No counterpart
   in the reference, whose HDoG3D_main runs its substacks one at a time
   (src/3D/HDoG3D_main.cpp:294-315); the records are the ones hdog_run_stack gives each stack.
   The caller gives one context per frame shape (width x height; at most 64 substacks each)
   and the stacks in device memory.  hdog_graph_create schedules every stack's substacks
   (HDoG3D_main's schedule), picks each frame shape's launch shapes with the autotuner on its
   first batch, packs each shape's substacks into batches of its context, and captures all
   batches of all shapes into one CUDA graph: the two sweeps run as persistent kernels over a
   device work queue of (substack, tile) items when the autotuner chose that, the records
   of every batch are placed in one device array of the run, and nothing returns to the host
   between batches.  hdog_graph_run launches the graph and returns the records stack by stack
   in the caller's order (stack_counts[i], may be NULL, receives stack i's count); when a
   batch needs the host's fallback (a full foreground list or region table, or more records
   than the run's array holds) it reruns the stacks one by one without the graph, with the
   same results.  The graph keeps the stacks' device addresses and the contexts' scratch: the
   stacks must stay in place, and the contexts are locked while the graph runs. */
typedef struct hdog_graph_stack {
  const uint16_t *data;   /* device memory: length slices of width * height uint16 */
  int width, height, length;
} hdog_graph_stack;
typedef struct hdog_graph hdog_graph;
int hdog_graph_create(hdog_ctx *const *ctxs, int n_ctx, const hdog_graph_stack *stacks, int n_stacks, void *stream,
                      hdog_graph **out);
int hdog_graph_run(hdog_graph *g, hdog_record *out, int64_t cap, int64_t *n_records, int64_t *stack_counts,
                   void *stream);
/* The records of the graph's last run (also after HDOG_ERR_CAPACITY). */
int hdog_graph_last_records(hdog_graph *g, hdog_record *out, int64_t cap, int64_t *n_records);
int hdog_graph_destroy(hdog_graph *g);

/* ---- autotuner ----
   Times the context's first batch of a device stack with each candidate launch shape of the
   two sweeps (one block per tile, or persistent grids of 3 / 2 DoG and 5 / 4 Hessian blocks
   per SM over the device work queue) and the full batch against half of it, keeps the
   fastest for the context (and for later contexts of the same frame shape, depth, radii and
   size in this process), and writes the timings as JSON for hdog_ctx_tuning.  No counterpart
   in the reference.  Every choice gives the same records. */
int hdog_autotune(hdog_ctx *ctx, const uint16_t *d_stack, int length, void *stream);
int hdog_ctx_tuning(hdog_ctx *ctx, char *buf, size_t cap);

/* ---- labelling without any device allocation ----
   No counterpart in the reference.  For callers that may not allocate device memory
   themselves (a host framework that owns all device memory through its own allocator,
   or a service with a fixed memory budget reserved at start-up): the same labels as
   hdog_ccl for a mask of at most 2^22 voxels (width * height * depth), with all scratch
   in one fixed 4.7 MB device array inside the library (per device, for the life of the
   process).  Larger volumes return HDOG_ERR_SHAPE.  Calls share that array: calls that
   overlap on the GPU (other streams or host threads) race; calls in sequence on one
   stream do not.  The first call on a device (and the first after a cudaDeviceReset,
   which gives the device a new context) looks up the array's device address with that
   device current; make that first call before any stream capture.  Synchronizes `stream`
   before returning. */
int hdog_ccl_noalloc(const uint8_t *d_mask, int32_t *d_labels, int width, int height, int depth,
                     void *stream);

/* ---- after the records: global coordinates, scale-merge validity, classifier features ----
   Per-record passes over record arrays in device memory (n may be 0), on `stream`
   (no synchronization).  The reference does these steps in NumPy on the host.

   Where a float64 scalar (a stack offset, a z bound) meets the float32 record fields the
   reference leaves the rounding to NumPy's promotion rules, which changed in NumPy 2: */
enum {
  HDOG_PROMOTE_F32 = 0,   /* NumPy 1.x value-based casting: the scalar is rounded to float32
                             and the arithmetic or comparison runs in float32 */
  HDOG_PROMOTE_F64 = 1    /* NumPy >= 2: float64 arithmetic or comparison, rounded to
                             float32 when stored into a float32 field */
};

/* dt_global of script/HalfBrainCells.py:16-20 and dt_scalemerged of script/MergeBrain.py:32-35,
   both packed (15 and 13 bytes), as NumPy lays them out. */
#pragma pack(push, 1)
typedef struct hdog_global {
  float merged_x, merged_y, merged_z;
  uint8_t i_x, i_y;
  uint8_t fwrv;                          /* 0 FW, 1 RV */
} hdog_global;
typedef struct hdog_scalemerged {
  float scaled_x, scaled_y, scaled_z;
  uint8_t is_valid;
} hdog_scalemerged;
#pragma pack(pop)

/* HDoGResultStack (script/HalfBrainCells.py:44-56): merged = offset + local * scale per axis
   (the scale a Python float, so the product is float32), and for a negative x (y) scale
   merged -= width * scale (height * scale).  i_x, i_y, fwrv are copied to every record. */
typedef struct hdog_global_params {
  double offset_x, offset_y, offset_z;   /* imagestack.offset_{x,y,z} (NumPy float64 scalars) */
  double scale_x, scale_y, scale_z;      /* coordinate_info.scale_{x,y,z} */
  int width, height;                     /* the stack's image size */
  int is_fw;                             /* 1: FW (fwrv 0), 0: RV (fwrv 1) */
  int i_x, i_y;                          /* stack grid position (stored as uint8) */
  int promote;                           /* HDOG_PROMOTE_* for offset + product */
} hdog_global_params;
int hdog_records_to_global(const hdog_record *d_records, int64_t n, const hdog_global_params *p,
                           hdog_global *d_out, void *stream);

/* process_stack of the scale-merge step (script/MergeBrain.py:546-570): is_valid = z inside
   bound_z (either order, infinities allowed); scaled = A . ((merged - offset) * coeff -
   margin) + b, the inner expression stored as float32 and the affine step in float64. */
typedef struct hdog_scalemerge_params {
  double bound_z0, bound_z1;             /* bound_z (NumPy float64 scalars or +-inf) */
  double offset_x, offset_y, offset_z;   /* NumPy float64 scalars */
  double coeff_x, coeff_y, coeff_z;      /* downscale ratio / original scale (Python floats) */
  double margin_left, margin_top;        /* merged margins (Python ints) */
  double A[9];                           /* flip / axis permutation, row-major, entries 0 or +-1 */
  double b[3];
  int promote;                           /* HDOG_PROMOTE_* for merged - offset and the z test */
} hdog_scalemerge_params;
int hdog_scale_merge(const hdog_global *d_in, int64_t n, const hdog_scalemerge_params *p,
                     hdog_scalemerged *d_out, void *stream);

/* get_X_3d (script/HDoG_classifier.py:158-176): X = nan_to_num((log10(F + bias_before_log) +
   bias) * scale) in float64, F = (intensity, structureness, blobness) of each record
   (intensity / size when is_ave).  X is n x 3, row-major.  log10 is CUDA's (at most 1 ulp
   from the correctly rounded value, as the host libm's is within its own bound). */
typedef struct hdog_clf_params {
  double bias[3];                        /* default 0 */
  double scale[3];                       /* default 1 */
  double bias_before_log[3];             /* default 0 */
  int is_ave;
} hdog_clf_params;
int hdog_classifier_features(const hdog_record *d_records, int64_t n, const hdog_clf_params *p, double *d_X,
                             void *stream);

/* ---- the differentiable chain: normalize -> DoG -> Hessian -> relaxed mask score ----
   Float32 forward and hand-written adjoint (no counterpart in the reference, whose chain
   is not differentiable).  The stages follow the detection path's borders
   (NormalizeFilter.cu:537-654, DoG3DFilter.cu:70-437, Hessian3DFilter_element.cu:22-388)
   without its bit-exact summation orders; each axis and scale has its own sigma; the mask
   test xx < 0, xx yy - xy^2 > 0, det < 0 (Hessian3DFilter_element.cu:317-321) becomes
   sigmoid((b0 - xx) / tau) * sigmoid((xx yy - xy^2 - b1) / tau^2) * sigmoid((b2 - det) / tau^3)
   with thresholds b (zero: the reference's test).  Loss = mean score at the positive points -
   mean score at the negative points.  Points are int32 (z, y, x) triples.  Backward
   recomputes the forward from the input and returns d loss / d volume, d loss / d sigma and
   d loss / d thresholds (any may be NULL);
   tap radii (int)(2 sigma + 0.5) are held fixed for the derivatives.  Sigmas up to 15.7
   (radius 31).  The workspace is device memory of hdog_soft_workspace_bytes bytes. */
typedef struct hdog_soft_params {
  int width, height, depth;
  int radius_norm_xy, radius_norm_z;
  float min_intensity;
  float sigma[6];                        /* x1, y1, z1 (small scale), x2, y2, z2 (large scale) */
  float gamma;                           /* normalizer (sx1 sy1 sz1)^gamma */
  float tau;                             /* scale of the relaxed minor tests (> 0) */
  float thresh[3];                       /* b0, b1, b2: offsets of the three minor tests */
} hdog_soft_params;
size_t hdog_soft_workspace_bytes(const hdog_soft_params *p);
int hdog_soft_forward(const hdog_soft_params *p, const float *d_volume, const int32_t *d_pos, int n_pos,
                      const int32_t *d_neg, int n_neg, float *d_loss, float *d_scores, void *d_workspace,
                      void *stream);
int hdog_soft_backward(const hdog_soft_params *p, const float *d_volume, const int32_t *d_pos, int n_pos,
                       const int32_t *d_neg, int n_neg, float grad_loss, float *d_grad_volume,
                       float *d_grad_sigma, float *d_grad_thresh, void *d_workspace, void *stream);
/* hdog_soft_backward that takes the forward chain's intermediates (min / max and box-mean
   volumes, normalized volume, DoG) from d_workspace instead of recomputing them: the
   workspace must be the one an hdog_soft_forward call filled with the same parameters and
   volume, with nothing else written to it since (backward calls leave those parts intact, so
   several may follow one forward).  Same results as hdog_soft_backward. */
int hdog_soft_backward_kept(const hdog_soft_params *p, const float *d_volume, const int32_t *d_pos, int n_pos,
                            const int32_t *d_neg, int n_neg, float grad_loss, float *d_grad_volume,
                            float *d_grad_sigma, float *d_grad_thresh, void *d_workspace, void *stream);

/* ---- context options ---- */
enum {
  HDOG_OPT_FUSED_SWEEP = 1,  /* 1 (default): DoG, Hessian and the PD test in one z-sweep kernel
                                when the radii allow; 0: separate passes (same results) */
  HDOG_OPT_HOST_BATCH = 2,   /* substacks in the first batch when hdog_run_stack gets its stack
                                in host memory (default 1; 0: as many as the context holds);
                                each later batch holds at most twice as many as the one before
                                (and at most what the context holds): the stack is copied in
                                chunks on a second stream and each batch waits only for its own
                                slices, so the copy of each chunk overlaps the batch before it.
                                Records are the same for every value. */
  HDOG_OPT_WALK_LIMIT = 3    /* bound of the labelling's union-find walks and link retries
                                (default 0: the substack's voxel count, which no walk reaches).
                                A smaller bound makes a walk that passes it give up and the call
                                return HDOG_ERR_TIMEOUT instead of running on; the context stays
                                usable.  For tests of that error path. */
};
int hdog_ctx_set_option(hdog_ctx *ctx, int option, int value);

/* ---- diagnostics ----
   Cross-tile edges the last labelling of the context's first substack produced, and the
   edge list's capacity; above it the labelling merged those edges from the mask instead.
   No counterpart in the reference (its CCL has no edge list).  Synchronizes the device. */
int hdog_ccl_edge_count(hdog_ctx *ctx, int64_t *edges, int64_t *capacity);

/* ---- per-kernel timing (CUDA events on the launching stream) ---- */
/* When on, every kernel launch of the context's calls is bracketed by two events. */
int hdog_timing_enable(hdog_ctx *ctx, int on);
/* Writes "kernel_name launches total_ms\n" lines accumulated since the last read
   (waiting for the recorded events), then resets the accumulators.  Names starting with
   "host_" are wall times of host phases of the whole-chain calls (enqueueing a batch,
   waiting for it, collecting its records, waiting for a host stack's chunk, the final copy
   to the caller's buffer). */
int hdog_timing_read(hdog_ctx *ctx, char *buf, size_t cap);

/* ---- small helpers for bindings without a CUDA runtime of their own ---- */
int hdog_memcpy(void *dst, const void *src, size_t bytes, void *stream);  /* cudaMemcpyDefault */
int hdog_stream_sync(void *stream);
int hdog_device_alloc(void **ptr, size_t bytes);
int hdog_device_free(void *ptr);

#ifdef __cplusplus
}
#endif
#endif
