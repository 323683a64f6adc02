/*
 * autoscoper_gb300.h -- C ABI of the GB300-native registration cost path.
 *
 * Drop-in boundary for Autoscoper's CUDA backend (namespace xromm::gpu in
 * libautoscoper/src/gpu/cuda).  Every entry point returns an int status
 * (ASC_OK = 0, negative on error) instead of exiting the process; none
 * falls back to the CPU.  Image buffers are device float32 arrays, row-major
 * with row stride = width, owned by the caller exactly as in the reference
 * (Tracker.cpp:292-298).  `stream` is a cudaStream_t (NULL = legacy default
 * stream); every call is asynchronous on it unless stated otherwise.
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the reference project root).  The C++ classes with the
 * reference's own signatures are in autoscoper_gb300.hpp.
 */
#ifndef AUTOSCOPER_GB300_H
#define AUTOSCOPER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASC_OK 0
#define ASC_ERR_ARG -1        /* bad argument (null pointer, size, kind) */
#define ASC_ERR_CUDA -2       /* a CUDA runtime call failed */
#define ASC_ERR_EMPTY -3      /* empty volume (reference: exit(0)) */
#define ASC_ERR_RANGE -4      /* size beyond a buffer or a fixed limit */
#define ASC_ERR_NOMEM -5      /* device allocation failed or over budget */
#define ASC_ERR_TIMEOUT -6    /* a bounded device wait gave up */
#define ASC_ERR_STATE -7      /* call out of order (e.g. no volume set) */

/* Volume storage formats on the device (sampled in FP32 in every case). */
#define ASC_STORE_U16 0   /* integer voxels as stored (u8/u16 input) */
#define ASC_STORE_F16 1   /* voxels rounded to IEEE half */
#define ASC_STORE_BF16 2  /* voxels rounded to bfloat16 */
#define ASC_STORE_F32 3   /* voxels as FP32: twice the bytes, no unpacking in the march */

/* NCC/SAD coverage: the reference's sum() (Ncc_kernels.cu:151-187) folds
 * each level's shared memory with s = T/2, T/4, ... and so drops partials
 * whenever a level's thread count T is not a power of two.  ASC_SUM_TREE
 * reproduces that coverage exactly; ASC_SUM_FULL sums every pixel. */
#define ASC_SUM_TREE 0
#define ASC_SUM_FULL 1

typedef struct asc_volume_s *asc_volume;
typedef struct asc_image_s *asc_image;
typedef struct asc_engine_s *asc_engine;

/* Options (asc_set_option).  ASC_OPT_EMPTY_SKIP (default 1): the ray march
 * steps over runs of samples inside 8^3-voxel cells whose voxels are all at
 * or below the cutoff.  Such samples add exactly nothing in the reference
 * (RayCaster_kernels.cu:189), so results are identical either way; 0 reads
 * every sample (for A/B checks). */
#define ASC_OPT_EMPTY_SKIP 1
int asc_set_option(int option, int value);

const char *asc_version(void);
const char *asc_status_string(int status);
/* Last CUDA error text seen by the library on this thread ("" if none). */
const char *asc_last_error(void);

/* ---- device memory helpers ----
 * replaces gpu::cudaMallocWrap (libautoscoper/src/gpu/cuda/CudaWrap.cpp:59-62) */
int asc_malloc(void **ptr, size_t bytes);
int asc_free(void *ptr);
int asc_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream);
int asc_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream);
/* Device to device, asynchronous: View::filter's copy for an empty or
 * disabled filter (View.cpp:479-483, :500-517). */
int asc_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream);
int asc_memset(void *dst, int value, size_t bytes, void *stream);
int asc_stream_sync(void *stream);
int asc_device_sync(void);
/* Plumbing for callers without their own CUDA runtime bindings (the ctypes
 * layer, benchmarks): device selection, streams, events, pinned host memory. */
int asc_set_device(int device);
int asc_stream_create(void **stream);
int asc_stream_destroy(void *stream);
int asc_event_create(void **event);
int asc_event_record(void *event, void *stream);
int asc_event_elapsed(void *start, void *stop, float *ms);
int asc_event_destroy(void *event);
int asc_host_alloc(void **ptr, size_t bytes);
int asc_host_free(void *ptr);
/* Free and total device memory of the current device (cudaMemGetInfo). */
int asc_mem_info(size_t *free_bytes, size_t *total_bytes);
/* Read bandwidth of the current device, the denominator of the benchmark's
 * roofline fractions (no counterpart in the reference): a buffer of `bytes`
 * (allocated and freed here) is streamed with 16-byte loads that bypass L1,
 * once to warm up and then `passes` times in one timed launch.  A buffer
 * well inside L2 measures L2 read bandwidth, one far larger than L2 HBM.
 * gbs: 1e9 bytes/s read; ms (optional): the timed launch.  Blocking. */
int asc_probe_read_bandwidth(size_t bytes, int passes, double *gbs, float *ms);

/* ---- volumes ----
 * replaces gpu::VolumeDescription::VolumeDescription(const Volume&)
 * (libautoscoper/src/VolumeDescription.cpp:152-305): flips, crops to the
 * non-zero box, records min/max and the normalisation constants, uploads.
 * data: width*height*depth voxels (x fastest), bps 8 or 16; scale: voxel
 * size in mm; flip: 0/1 per axis; storage: ASC_STORE_*.  A cropped volume of
 * 2^31 voxels or more (its two-voxel padding included) is ASC_ERR_RANGE. */
int asc_volume_create(const void *data, int width, int height, int depth, int bps, const double scale[3],
                      const int flip[3], int storage, asc_volume *out);
/* invScale(), invTrans(), transCenter(), minValue(), maxValue() and the
 * cropped dimensions (VolumeDescription.hpp:63-70). */
int asc_volume_info(asc_volume vol, float inv_scale[3], float inv_trans[3], double trans_center[3],
                    float *min_value, float *max_value, int dims[3]);
int asc_volume_destroy(asc_volume vol);

/* ---- DRR ray caster ----
 * replaces RayCaster::setInvModelView + setViewport + render
 * (libautoscoper/src/gpu/cuda/RayCaster.cpp:88-143) and volume_render
 * (RayCaster_kernels.cu:81-104).  inv_model_view: the 16 doubles of
 * CoordFrame::to_matrix_row_order of the camera->volume frame (the
 * normalisation is folded in here, as setInvModelView does);
 * viewport: (x, y, width, height) on the film plane; visible = 0 clears. */
int asc_raycast(asc_volume vol, const double inv_model_view[16], const float viewport[4], float sample_distance,
                float ray_intensity, float cutoff, int visible, float *out, int width, int height, void *stream);

/* ---- radiograph and background samplers ----
 * replaces RadRenderer::set_rad (RadRenderer.cpp:81-105) and
 * BackgroundRenderer::set_back (BackgroundRenderer.cpp:74-86): an image held
 * on the device.  bps: 8 or 16 (radiograph, normalized) or 32 (float32
 * background, read as stored). */
int asc_image_create(const void *data, int width, int height, int bps, asc_image *out);
/* Replaces the pixels of an image of the same size (the per-frame
 * Video::set_frame + set_rad of Tracker::optimize, Tracker.cpp:381-386)
 * without reallocating; asynchronous on `stream`. */
int asc_image_update(asc_image img, const void *data, void *stream);
int asc_image_destroy(asc_image img);
/* RadRenderer::render (RadRenderer.cpp:123-142, image_render_kernel
 * RadRenderer_kernels.cu:85-116): out = 1 - bilinear(rad) inside the
 * image plane, 0 outside.  image_plane = the camera viewport. */
int asc_rad_render(asc_image img, const float image_plane[4], const float viewport[4], float *out, int width,
                   int height, void *stream);
/* BackgroundRenderer::render (BackgroundRenderer.cpp:88-124): out =
 * (threshold <= bilinear(bg)) ? 1 : 0 inside, 0 outside. */
int asc_background_render(asc_image img, const float image_plane[4], const float viewport[4], float threshold,
                          float *out, int width, int height, void *stream);

/* ---- elementwise ----
 * drr_background (DRRBackground_kernels.cu:47-75), multiply
 * (Mult_kernels.cu:49-77), merge (Merger_kernels.cu:49-75), composite
 * (Compositor_kernels.cu:53-88; writes 3*w*h interleaved RGB), fill
 * (Compositor_kernels.cu:64-68; this one honours `value`, the reference
 * always writes 1.0). */
int asc_drr_background(const float *src, float *dst, int width, int height, void *stream);
int asc_multiply(const float *a, const float *b, float *dst, int width, int height, void *stream);
int asc_merge(const float *a, const float *b, float *dst, int width, int height, void *stream);
int asc_composite(const float *a, const float *b, const float *c, const float *d, float *dst, int width, int height,
                  void *stream);
int asc_fill(float *dst, size_t count, float value, void *stream);
/* Video::create_background_image (Video.cpp:147-218): out (device, w*h
 * floats) = per pixel the largest normalized value of n >= 2 frames (8 or
 * 16 bits per sample, all of one size). */
int asc_background_from_frames(const asc_image *frames, int n, float *out, void *stream);

/* ---- filters ----
 * SobelFilter::apply (SobelFilter_kernels.cu:63-113), ContrastFilter::apply
 * (ContrastFilter_kernels.cu:62-96), GaussianFilter::apply
 * (GaussianFilter.cpp:73-134, GaussianFilter_kernels.cu:61-97),
 * SharpenFilter::apply (SharpenFilter.cpp:58-158, SharpenFilter_kernels.cu:74-129).
 * in and out must not alias.  A Gaussian/Sharpen radius with
 * 2*floor(3r)+1 == 1 copies the image. */
int asc_sobel(const float *in, float *out, int width, int height, float scale, float blend, void *stream);
int asc_contrast(const float *in, float *out, int width, int height, float alpha, float beta, int size,
                 void *stream);
int asc_gaussian(const float *in, float *out, int width, int height, float radius, void *stream);
int asc_sharpen(const float *in, float *out, int width, int height, float radius, float contrast, float threshold,
                void *stream);

/* ---- cost reductions ----
 * replaces gpu::ncc_init / ncc (Ncc_kernels.cu:87-134) and gpu::hdist_init /
 * hdist (HDist_kernels.cu:50-134).  asc_ncc_init(max_n) sizes the per-block
 * partial buffer used by asc_ncc/asc_hdist (max_n = 0 frees it).  The result
 * is written to *result_dev (a device double) without a host sync; NCC
 * keeps the reference's 1e5 value for a denominator below 1e-5.
 * `coverage` is ASC_SUM_TREE or ASC_SUM_FULL. */
int asc_ncc_init(unsigned max_n);
int asc_ncc(const float *f, const float *g, const float *mask, unsigned n, int coverage, double *result_dev,
            void *stream);
int asc_hdist(const float *f, const float *g, const float *mask, unsigned n, int coverage, double *result_dev,
              void *stream);
/* NCC that allocates nothing.  No counterpart in the reference: for callers
 * that cannot allocate device memory when they score (an application that
 * owns a fixed device-memory budget and does not let a library grow it, or a
 * latency-critical loop that cannot afford cudaMalloc's implicit device
 * synchronisation).  Same arguments, kernel and result as asc_ncc, but the
 * per-block partials live in a fixed array compiled into the library, which
 * every GPU that loads the library holds until exit (about 288 KiB).
 * n may be at most ASC_NOALLOC_MAX_N elements; larger n returns
 * ASC_ERR_RANGE.  The first call on a device looks up the array's device
 * address, so make that first call before any stream capture; the address is
 * kept per CUDA context, so after a cudaDeviceReset the next call (again
 * outside any capture) looks it up anew.  All calls on
 * a device share the array: calls that overlap on the GPU (different
 * streams, or a second call issued before the first has finished on another
 * stream) race and must be serialised by the caller. */
#define ASC_NOALLOC_MAX_N (1u << 24)
int asc_ncc_noalloc(const float *f, const float *g, const float *mask, unsigned n, int coverage,
                    double *result_dev, void *stream);
/* Blocking convenience forms returning the value on the host (the
 * reference's float ncc(...) / hdist(...) signatures). */
int asc_ncc_host(const float *f, const float *g, const float *mask, unsigned n, int coverage, double *result,
                 void *stream);
int asc_hdist_host(const float *f, const float *g, const float *mask, unsigned n, int coverage, double *result,
                   void *stream);

/* ---- batched registration engine (Tracker::minimizationFunc batched) ----
 * An engine holds a scene resident on the device: cameras, volumes,
 * radiographs, filter chains, ray-caster settings, pivots and base poses.
 * asc_engine_eval scores many (bone, manipulator) candidates in one pass of
 * fused launches; see asc_engine.h-level docs in autoscoper_gb300.hpp. */
typedef struct {
  int kind;          /* 0 contrast, 1 sobel, 3 gaussian, 4 sharpen (Filter.hpp:59-66) */
  int enabled;
  float p0, p1, p2;  /* sobel: scale, blend; contrast: alpha, beta, size;
                        gaussian: radius; sharpen: radius, contrast, threshold */
} asc_filter_desc;

typedef struct {
  double frame[12];       /* camera -> world CoordFrame (rotation columns, translation) */
  double viewport[4];     /* Camera::viewport() */
  double image_plane[12]; /* Camera::image_plane() */
  asc_image radiograph;   /* current frame's radiograph */
  asc_image background;   /* optional float image (NULL = none) */
  float bg_threshold;     /* < 0 disables the background mask (View.cpp:171-194) */
  int n_drr_filters, n_rad_filters;
  asc_filter_desc drr_filters[8];
  asc_filter_desc rad_filters[8];
} asc_view_desc;

typedef struct {
  asc_volume volume;
  double pivot[12];       /* volume matrix (Trial::getVolumeMatrix after the pivot translate) */
  double base_pose[6];    /* current pose xyzypr (the values the reference reads from its curves) */
  float step[4], intensity[4], cutoff[4];  /* RayCaster settings per view */
} asc_bone_desc;

/* cf_model (Tracker::optimize's cf_model, Tracker.cpp:762-770): 0 scores a
 * view by 1 - NCC, 1 by the SAD of gpu::hdist (HDist_kernels.cu:111-203).
 * Up to 16 views and 64 bones; each bone is scored in the first
 * min(n_views, 4) views (asc_engine_set_bone picks others). */
int asc_engine_create(int n_views, const asc_view_desc *views, int n_bones, const asc_bone_desc *bones,
                      int render_width, int render_height, int max_items, int coverage, int cf_model,
                      asc_engine *out);
int asc_engine_destroy(asc_engine e);
int asc_engine_set_base_pose(asc_engine e, int bone, const double xyzypr[6]);
int asc_engine_set_radiograph(asc_engine e, int view, asc_image radiograph);
/* Serving: an engine's views and bones as slots that hold different jobs
 * over its lifetime (no counterpart in the reference, which holds one trial).
 * asc_engine_set_view replaces view `view` (camera, radiograph, background,
 * filter lists) and gives it its own render size (at most the engine's);
 * asc_engine_set_bone replaces bone `bone` (volume, pivot, base pose) and
 * scores it in engine views views[0 .. n_views) with desc->step/intensity/
 * cutoff[j] in views[j] (n_views at most min(the engine's views, 4)).  A
 * candidate of a bone is then scored in that bone's views only, so one batch
 * mixes bones of different jobs (cameras, radiographs, filters, render sizes).
 * Call between evaluations (they copy to the device synchronously); engines
 * with bones moved to other views serve asc_engine_eval / _eval_host and the
 * optimizers, and their plain path and image exports return ASC_ERR_STATE.
 * view_cost outputs hold min(n_views of the engine, 4) entries per candidate,
 * in the order of the bone's views, 0 past its last. */
int asc_engine_set_view(asc_engine e, int view, const asc_view_desc *desc, int render_width, int render_height);
int asc_engine_set_bone(asc_engine e, int bone, const asc_bone_desc *desc, int n_views, const int *views);
/* Launch shapes of an engine's evaluation (no counterpart in the
 * reference): blocks per SM of the ray-cast kernel (1..4) and of the
 * filter/NCC kernel (0: as many as fit), and the ray block each warp of a
 * 16 x 16 ray tile takes (2: 4 x 8 rays, 3: 8 x 4, 4: 16 x 2).  Results do
 * not depend on them.  asc_engine_create applies the loaded tuning table's
 * entry for the engine's workload class (asc_engine_workload_class: ceil
 * log2 of the render pixels, ceil log2 of the largest volume's voxels, the
 * views), else the defaults {4, 0, 3}.  asc_tuning_load reads the table the
 * project's autotuner writes (autoscoper_gb300/tuning.txt: lines of
 * "rpx vox views ray_blocks view_blocks ray_shape", '#' comments) and
 * replaces the loaded one; engines created before keep their shapes. */
typedef struct {
  int ray_blocks_per_sm;
  int view_blocks_per_sm;
  int ray_shape;
} asc_launch_config;
int asc_engine_set_launch(asc_engine e, const asc_launch_config *cfg);
int asc_engine_get_launch(asc_engine e, asc_launch_config *cfg, int *view_blocks_max);
int asc_engine_workload_class(asc_engine e, int out[3]);
int asc_tuning_load(const char *path);
/* RayCaster::setVisible for one bone in every view (the volume visibility
 * of AutoscoperMainWindow::setVolumeVisibility): a hidden bone renders an
 * all-zero DRR, so its views score the empty-mask cost. */
int asc_engine_set_visible(asc_engine e, int bone, int visible);
/* Scores n candidates: bone[i] and manip[6*i] (xyz mm + axis-angle degrees,
 * CoordFrame::from_xyzAxis_angle).  cost_dev (device, n doubles) receives
 * minimizationFunc's value; view_cost_dev (optional, n*n_views) the per-view
 * terms of trackFrame.  Inputs are device pointers. */
int asc_engine_eval(asc_engine e, int n, const int *bone_dev, const double *manip_dev, double *cost_dev,
                    double *view_cost_dev, void *stream);
/* Host-pointer form: copies the candidates in and the costs out (blocking). */
int asc_engine_eval_host(asc_engine e, int n, const int *bone, const double *manip, double *cost,
                         double *view_cost, void *stream);
/* The plain per-pose drop-in form of the same evaluation: for each candidate,
 * Tracker::trackFrame's call sequence (Tracker.cpp:603-770) over the plain
 * per-operator kernels above, with the NCC read back to the host after every
 * view as the reference does.  Host pointers; blocking. */
int asc_engine_eval_plain(asc_engine e, int n, const int *bone, const double *manip, double *cost,
                          double *view_cost, void *stream);
/* Device pointers of the last evaluation's DRR images and per-item-view
 * layout, for inspection/tests: layout[5*k] = (ok, width, height, offset, tiles). */
int asc_engine_debug(asc_engine e, const float **drr_dev, const int **layout_dev);
/* Instrumentation of asc_engine_eval: with profiling on, events bracket the
 * set-up, ray-cast and view kernels of each evaluation; stats returns the
 * last evaluation's phase times (ms) and its trilinear sample and pixel
 * counts (the work figures of the roofline). */
int asc_engine_profile(asc_engine e, int enable);
int asc_engine_stats(asc_engine e, float ms[3], unsigned long long *samples, unsigned long long *pixels);
/* Ray-cast work counters of the last evaluation: out[0] trilinear samples of
 * the reference's march (far to near over the whole box), out[1] pixels,
 * out[2] samples actually marched after empty-space skipping, out[3] lane
 * slots the marching warps occupied (32 x the longest marched span of each
 * warp's rays); out[2] / out[3] is the SIMT efficiency of the march. */
int asc_engine_counters(asc_engine e, unsigned long long out[4]);
/* Rays of the last evaluation that the ray cast marched a second time: rays
 * with a sample whose FP32 value lay within rounding of the cutoff, whose
 * decision (RayCaster_kernels.cu:190, sample > cutoff) was then made from a
 * double-float position and value, so that every DRR pixel counts the same
 * samples as an exact computation.  No counterpart in the reference. */
int asc_engine_exact_rays(asc_engine e, int *n);

/* ---- device-resident optimizers ----
 * Synchronous batched PSO over all bones at once: n_particles per bone,
 * n_iter iterations; inertia w, c1, c2; particles start uniform in
 * [lo, hi]^6 (particle 0 at the zero manipulator, PSO.cpp:207-214).  Each
 * iteration (velocity/position update, scoring, best updates) is one CUDA
 * graph launch.  best_manip (host, 6 per bone) and best_cost (host, per
 * bone) receive gBest.  evals_out (optional) the number of poses scored. */
int asc_engine_pso(asc_engine e, int n_particles, int n_iter, double w, double c1, double c2, double lo, double hi,
                   uint64_t seed, double *best_manip, double *best_cost, long long *evals_out, void *stream);
/* asc_engine_pso with the stall rule of pso() (PSO.cpp:271-285) per bone:
 * after each iteration a gBest change below 1e-4 counts a stall, one above
 * 1e-3 resets the count; max_stall stalls in a row stop that bone's swarm,
 * and the iterations end when every swarm has stopped or after n_iter
 * (max_stall 0: never stalls).  iterations_out (optional): iterations run. */
int asc_engine_pso_stall(asc_engine e, int n_particles, int n_iter, int max_stall, double w, double c1, double c2,
                         double lo, double hi, uint64_t seed, double *best_manip, double *best_cost,
                         long long *evals_out, int *iterations_out, void *stream);

/* Many Nelder-Mead simplices in lock-step (AMOEBA, DownhillSimplex.cpp:39-172):
 * each iteration evaluates, per simplex, the reflection and speculatively the
 * expansion and both contraction points in one batch call, then applies
 * AMOEBA's decision rules, so each simplex follows the sequential AMOEBA's
 * trajectory exactly.  P: ns x (ndim+1) x ndim, Y: ns x (ndim+1) (in/out);
 * cost(n, who, x, y, ctx) fills y[i] for point x[i*ndim..] of simplex who[i]. */
typedef int (*asc_batch_cost_fn)(int n, const int *who, const double *x, double *y, void *ctx);
int asc_amoeba_batch(asc_batch_cost_fn cost, void *ctx, int ns, double *P, double *Y, int ndim, double ftol,
                     int *iterations);

/* Tracker::optimize (Tracker.cpp:337-580) for one frame and every bone of
 * an engine at once.  method 0: PSO (asc_engine_pso with the parameters
 * below), the pose moved to the swarm's best, then Downhill Simplex from the
 * offsets; method 1: Downhill Simplex only.  As in the reference, the
 * simplex result is kept only if it beats the cost at the frame's start pose
 * (method 0).  Poses are rounded to float as the reference's key curves store
 * them.  The engine's base poses are updated; pose_out (6 per bone) and
 * cost_out (per bone) receive them. */
typedef struct {
  int method;          /* 0 PSO + simplex, 1 simplex only */
  int n_particles, n_iter;
  double w, c1, c2, lo, hi;
  uint64_t seed;
  double offsets[6];   /* initial simplex offsets (Trial::offsets, default 0.1) */
  double ftol;         /* 1e-3 in the reference */
  int max_stall;       /* PSO stall limit (asc_engine_pso_stall); 0: n_iter iterations */
} asc_opt_params;
int asc_engine_optimize_frame(asc_engine e, const asc_opt_params *params, double *pose_out, double *cost_out,
                              long long *evals_out, void *stream);
/* asc_engine_optimize_frame that also returns, per bone, the pose before the
 * key curves store it (raw_out, 6 per bone: the xyzypr Tracker::optimize
 * inserts into its curves, Tracker.cpp:558-571). */
int asc_engine_optimize_frame_ex(asc_engine e, const asc_opt_params *params, double *pose_out, double *raw_out,
                                 double *cost_out, long long *evals_out, void *stream);

/* View::renderDrr (View.cpp:201-231) on an engine's view: the DRRs of all
 * bones at poses (n_bones x 6 xyzypr) over `viewport` (NULL: the whole
 * image, (-w/2, -h/2, w, h) of the camera viewport), summed and clamped to 1,
 * then the view's DRR filters.  out: device floats of the render size
 * (viewport size x render size / camera viewport, at most the engine's). */
int asc_engine_render_drr(asc_engine e, int view, const double *poses, const double *viewport, float *out,
                          void *stream);
/* Tracker::getImageData (Tracker.cpp:865-925): bone `bone` at `pose` over
 * the whole image at the engine's render size: the filtered radiograph, the
 * filtered DRR and the mask (background x DRR mask), the first two masked.
 * rad, drr, mask: device floats (render width x height, reported). */
int asc_engine_image_data(asc_engine e, int view, int bone, const double pose[6], float *rad, float *drr,
                          float *mask, int *width, int *height, void *stream);

/* The pose a trial's key curves hold after Tracker::optimize stores `pose`
 * (xyzypr) and reads it back (Tracker.cpp:422-438, KeyCurve<float> and
 * KeyCurve<Quatf>): x, y, z rounded to float, the rotation through a float
 * quaternion.  Host arithmetic only. */
int asc_keycurve_store(const double pose[6], double out[6]);

/* A volume's pose curves over frames (Trial::getXCurve/.../getQuatCurve):
 * x, y, z as KeyCurve<float> (cubic segments between keys with SMOOTH
 * tangents, KeyCurve.hpp:231-446) and the rotation as KeyCurve<Quatf>
 * (slerp between keys, Quaternion.hpp:380-403).  insert stores a pose at a
 * frame in the curves named by `mask` as AutoscoperMainWindow::setPose does
 * (x, y, z as float; Quatf(yaw, pitch, roll)); erase removes their keys at a
 * frame; eval reads the pose at a frame as getPose does (the curves'
 * values, the rotation's toEuler as yaw, pitch, roll); keys reports which
 * curves hold a key at a frame.  Host arithmetic only. */
typedef struct asc_pose_curve_s *asc_pose_curve;
#define ASC_CURVE_X 1
#define ASC_CURVE_Y 2
#define ASC_CURVE_Z 4
#define ASC_CURVE_ROT 8
#define ASC_CURVE_ALL 15
int asc_pose_curve_create(asc_pose_curve *out);
int asc_pose_curve_destroy(asc_pose_curve c);
int asc_pose_curve_clear(asc_pose_curve c);
int asc_pose_curve_insert(asc_pose_curve c, int frame, const double xyzypr[6], int mask);
int asc_pose_curve_erase(asc_pose_curve c, int frame, int mask);
int asc_pose_curve_keys(asc_pose_curve c, int frame, int *mask);
int asc_pose_curve_eval(asc_pose_curve c, int frame, double xyzypr[6]);
/* A pose as the 4 x 4 column-major matrix of its CoordFrame (from_xyzypr
 * then to_matrix, CoordFrame.cpp:100-108, :203-221) and back (from_matrix
 * then to_xyzypr, :177-201): the tracking files' matrix form. */
int asc_pose_to_matrix(const double xyzypr[6], double m[16]);
int asc_pose_from_matrix(const double m[16], double xyzypr[6]);

/* A sequence of Tracker::optimize calls (Tracker.cpp:337-580), frames in
 * order (dframe +1) or in reverse (dframe -1).  Per frame: the views take
 * the frame's radiographs rads[frame * n_views + view]; the start pose is
 * the previous tracked frame's pose stored anew (guess 1, from the second
 * tracked frame on), the linear extrapolation of the two previous tracked
 * frames (guess 2, from the third on), or else the frame's key-curve value:
 * poses[frame] for the first frame and for frames marked in `keyed`, the
 * previous tracked frame's pose for the others (a curve holds its last key
 * beyond it); then `repeats` times asc_engine_optimize_frame from the
 * frame's pose.  poses: n_frames x n_bones x 6 (in: the key-curve values;
 * out: the tracked poses); costs (optional): n_frames x n_bones. */
typedef struct {
  asc_opt_params opt;
  int repeats;        /* >= 1 */
  int guess;          /* 0, 1 or 2 (Trial::guess) */
  int dframe;         /* +1 or -1 */
  const int *keyed;   /* n_frames flags: the frame holds a key (NULL: none but the first) */
} asc_track_params;
int asc_engine_track(asc_engine e, int n_frames, const asc_image *rads, const asc_track_params *params,
                     double *poses, double *costs, long long *evals_out, void *stream);

/* Tracker::optimize (Tracker.cpp:337-580) at one frame against each bone's
 * pose curves (curves: one asc_pose_curve per bone), with the views'
 * radiographs of that frame already set: the initial guess (params->guess 2:
 * CoordFrame::linear_extrap of the curves at frame - 2 dframe and
 * frame - dframe, when more than one frame lies behind in the dframe
 * direction; 1: the curves at frame - dframe, when one does) inserted at the
 * frame, then params->repeats times asc_engine_optimize_frame from the
 * curves' pose at the frame, the optimized pose inserted back.  n_frames:
 * the trial's frame count; keyed is not used.  costs (optional): per bone. */
int asc_engine_optimize_curves(asc_engine e, const asc_pose_curve *curves, int frame, int n_frames,
                               const asc_track_params *params, double *costs, long long *evals_out, void *stream);

/* Reference-sequential PSO on the host (PSO.cpp:198-295, asynchronous gBest,
 * glibc rand() after srand(seed), omega 0.8 * 0.9^epoch, c1 = c2 = 1.5),
 * with a caller-supplied cost.  Used to reproduce reference trajectories. */
typedef double (*asc_cost_fn)(const double *x, void *ctx);
int asc_pso_sequential(asc_cost_fn cost, void *ctx, int n_particles, float lo, float hi, unsigned max_epochs,
                       unsigned max_stall, unsigned seed, float best_pos[6], float *best_cost);
/* AMOEBA (DownhillSimplex.cpp:39-172) with a caller-supplied cost:
 * p = (ndim+1) x ndim vertices row-major, y = their values (in/out). */
int asc_amoeba(asc_cost_fn cost, void *ctx, double *p, double *y, int ndim, double ftol, int *iterations);

#ifdef __cplusplus
}
#endif

#endif
