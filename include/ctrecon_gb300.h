/*
 * ctrecon_gb300 -- C ABI of the GB300 (sm_103a) CT reconstruction hot path.
 *
 * Drop-in boundary for the filtered-backprojection / projection path of
 * CT_RECON_EXTENSIONS.  Every entry point replaces one GPU method of the
 * reference's operator API (the headers under its include/) with the same buffers and the
 * same meaning: the caller owns every buffer (input, output, geometry tables),
 * all pointers are device pointers unless stated otherwise, images are
 * [ny][nx] (row 0 on top), sinograms [na][ns] (view-major).
 *
 * Differences from the reference's GPU methods, by design:
 *   - the return value is a status code (CTR_OK == 0) instead of bool, and no
 *     C++ exception ever crosses this boundary;
 *   - work is stream-ordered on the given stream; entry points do not call
 *     cudaDeviceSynchronize (the C++ mirror classes in include/ct_recon/ add
 *     the blocking semantics of the reference methods);
 *   - results follow the reference's CPU code where its GPU code diverges
 *     (fan weighting offset and grad weight, single-view BP, ray-driven edge
 *     test);
 *   - *_f32 entry points compute in FP32 (geometry tables are read in FP64 and
 *     rounded once); *_f64 entry points compute in FP64.
 *
 * A batch of B independent items with the same geometry is passed with
 * `batch` = B; item b lives at in + b*in_size, out + b*out_size.
 */
#ifndef CTRECON_GB300_H
#define CTRECON_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ----------------------------------------------------- */
#define CTR_OK 0
#define CTR_ERR_INVALID_ARG 1  /* bad size, pointer, type or method       */
#define CTR_ERR_UNSUPPORTED 2  /* valid request this build does not handle */
#define CTR_ERR_CUDA 3         /* a CUDA runtime call failed               */
#define CTR_ERR_DEVICE 4       /* no sm_103 device / kernel image missing   */
#define CTR_ERR_KERNEL 5       /* a kernel reported an internal check       */

const char* ctr_status_string(int status);
/* Message of the last failing call on this host thread ("" if none). */
const char* ctr_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int ctr_version(void);
/* CTR_OK when the current device is a compute-capability 10.3 GPU that can
 * run this library's kernels. */
int ctr_device_check(void);
/* Reads (and optionally clears) the kernel self-check flags: bit 0 = a
 * detector window wider than its shared-memory slot, bit 1 = work-queue
 * overflow, bit 2 = a bounded wait gave up, bit 3 = a copy destination
 * failed its alignment check (the kernel then skips its work).  Synchronises
 * the device. */
int ctr_kernel_flags(unsigned int* flags, int reset);
/* Self-test of the bounded-wait error path (no counterpart in the reference,
 * whose GPU calls report failure as a false return after
 * cudaDeviceSynchronize, cuda/bp_fan_2d.cu:229-230): a one-CTA kernel waits,
 * with the same bounded mbarrier wait as the bulk-copy pipelines but a limit
 * of limit_ns (at most 1 s), for a copy that is never issued.  The wait runs
 * out, the kernel sets flag bit 2 and returns; the call returns
 * CTR_ERR_KERNEL and the context stays usable.  It leaves the flag set (read
 * and clear it with ctr_kernel_flags). */
int ctr_selftest_wait_timeout(unsigned long long limit_ns, cudaStream_t stream);

/* ---- parameter structs (field order of the reference Param structs) ---- */

/* FanWeightingParam, reference include/fan_weighting.h:21-39 */
typedef struct ctr_fan_weighting_param {
    unsigned int ns, nrow;
    double ds, offset, dso, dsd;
    int type; /* 1 "fan" (equiangular), 2 "flat" */
} ctr_fan_weighting_param;

/* FilterParam, reference include/filter.h:21-36 */
typedef struct ctr_filter_param {
    unsigned int ns, nrow;
    double ds, dsd;
    int type;   /* 0 "par", 1 "fan", 2 "flat" */
    int window; /* unused, as in the reference */
} ctr_filter_param;

/* FanBackprojection2DParam, reference include/bp_fan_2d.h:20-58 */
typedef struct ctr_fan_bp_param {
    unsigned int ns, na;
    double ds, orbit, offset_s, orbit_start;
    unsigned int nx, ny;
    double dx, dy, offset_x, offset_y, dso, dsd, fov;
} ctr_fan_bp_param;

/* FanBackprojection2DAngleParam, reference include/bp_fan_2d_angle.h:20-55 */
typedef struct ctr_fan_bp_angle_param {
    unsigned int ns, na;
    double ds, offset_s;
    unsigned int nx, ny;
    double dx, dy, offset_x, offset_y, dso, dsd, fov;
} ctr_fan_bp_angle_param;

/* ParallelBackprojection2DParam / ParallelSingleViewBp2DParam /
 * ParallelProjection2DParam (identical layouts), reference
 * include/bp_par_2d.h:20-55, include/bp_par_2d_sv.h:19-54,
 * include/fp_par_2d.h:20-55 */
typedef struct ctr_par_param {
    unsigned int ns, na;
    double ds, orbit, offset_s, orbit_start;
    unsigned int nx, ny;
    double dx, dy, offset_x, offset_y, fov;
} ctr_par_param;

/* ---- fan weighting: FanWeighting<T> / FanWeightingGrad<T>::calculate_on_gpu
 *      (reference include/fan_weighting.h:41-77).  in == out is allowed. ---- */
int ctr_fan_weighting_f32(const ctr_fan_weighting_param* p, const float* in, float* out,
                          int batch, cudaStream_t stream);
int ctr_fan_weighting_f64(const ctr_fan_weighting_param* p, const double* in, double* out,
                          int batch, cudaStream_t stream);
int ctr_fan_weighting_grad_f32(const ctr_fan_weighting_param* p, const float* in, float* out,
                               int batch, cudaStream_t stream);
int ctr_fan_weighting_grad_f64(const ctr_fan_weighting_param* p, const double* in,
                               double* out, int batch, cudaStream_t stream);

/* ---- ramp filter (reference include/filter.h:38-92) ----
 * filter: device double[2*ns+1], tap n at filter[n+ns] (RampFilterPrep).
 * RampFilter<T>: linear convolution out[r][i] = ds * sum_j in[r][j]*h[i-j];
 * RampFilterGrad<T>: the correlation (its adjoint).  in != out. */
int ctr_ramp_filter_prep(const ctr_filter_param* p, double* filter, cudaStream_t stream);
int ctr_ramp_filter_f32(const ctr_filter_param* p, const float* in, const double* filter,
                        float* out, int batch, cudaStream_t stream);
int ctr_ramp_filter_f64(const ctr_filter_param* p, const double* in, const double* filter,
                        double* out, int batch, cudaStream_t stream);
int ctr_ramp_filter_grad_f32(const ctr_filter_param* p, const float* in, const double* filter,
                             float* out, int batch, cudaStream_t stream);
int ctr_ramp_filter_grad_f64(const ctr_filter_param* p, const double* in,
                             const double* filter, double* out, int batch,
                             cudaStream_t stream);

/* ---- ramp filter on the BF16 tensor cores (no reference counterpart: the
 *      reduced-precision form of RampFilter<T> / RampFilterGrad<T>) ----
 * The filter as a dense Toeplitz GEMM, OUT = X * T^T with T[i][j] = ds*h[i-j]
 * (grad != 0: ds*h[j-i]).  X and T are split into `splits` BF16 terms and the
 * term products accumulate in FP32: splits = 2 (hi, lo; hi*hi + hi*lo +
 * lo*hi, 16 bits per operand) or 3 (hi, mid, lo; six products, 24 bits, the
 * accuracy of the FP32 filter on smooth sinograms, whose ramp filtering
 * cancels ~100x).  The input is stored as FP32, BF16 or FP16 (in_dtype); the optional
 * fan weighting (FanWeighting<T>, same ns) is applied to it first, in FP32.
 * The output is FP32 [batch*nrow][ns].  A plan owns the split T (built from
 * the device taps of ctr_ramp_filter_prep, on `stream`) and the split-X
 * workspace for max_batch sinograms; it serves one stream at a time. */
#define CTR_DTYPE_F32 0
#define CTR_DTYPE_BF16 1
#define CTR_DTYPE_F16 2
typedef struct ctr_ramp_tc_plan ctr_ramp_tc_plan;
int ctr_ramp_filter_tc_create(const ctr_filter_param* p, const double* filter,
                              const ctr_fan_weighting_param* weighting, int grad, int splits,
                              int max_batch, ctr_ramp_tc_plan** plan, cudaStream_t stream);
int ctr_ramp_filter_tc_run(ctr_ramp_tc_plan* plan, int in_dtype, const void* in, float* out,
                           int batch, cudaStream_t stream);
/* Device bytes the plan holds, and tensor-core FLOPs per input row (the term
 * products over the padded 128 x 64 tiles). */
int ctr_ramp_filter_tc_info(const ctr_ramp_tc_plan* plan, unsigned long long* workspace_bytes,
                            unsigned long long* mma_flops_per_row);
int ctr_ramp_filter_tc_destroy(ctr_ramp_tc_plan* plan);

/* ---- fan-beam pixel-driven backprojection, uniform orbit
 *      (reference include/bp_fan_2d.h:151-225) ----
 * Tables (FanBackprojection2DPixDrivenPrep / ...GradPrep): xpos double[nx],
 * ypos double[ny], sincostbl double[2*na] = (sin b, cos b) per view.
 * Forward: proj [na][ns] -> img [ny][nx], scaled by |orbit| / round(|na*orbit|/pi).
 * Grad: the exact adjoint, img [ny][nx] -> grad [na][ns]. */
int ctr_bp_fan_2d_prep(const ctr_fan_bp_param* p, double* xpos, double* ypos,
                       double* sincostbl, cudaStream_t stream);
int ctr_bp_fan_2d_f32(const ctr_fan_bp_param* p, const float* proj, float* img,
                      const double* xpos, const double* ypos, const double* sincostbl,
                      int batch, cudaStream_t stream);
int ctr_bp_fan_2d_f64(const ctr_fan_bp_param* p, const double* proj, double* img,
                      const double* xpos, const double* ypos, const double* sincostbl,
                      int batch, cudaStream_t stream);
int ctr_bp_fan_2d_grad_f32(const ctr_fan_bp_param* p, const float* img, float* grad,
                           const double* xpos, const double* ypos, const double* sincostbl,
                           int batch, cudaStream_t stream);
int ctr_bp_fan_2d_grad_f64(const ctr_fan_bp_param* p, const double* img, double* grad,
                           const double* xpos, const double* ypos, const double* sincostbl,
                           int batch, cudaStream_t stream);

/* ---- fan-beam backprojection with an explicit angle list
 *      (reference include/bp_fan_2d_angle.h:145-223) ----
 * angles: device double[na].  No output scale (the caller multiplies by the
 * orbit step, as the reference's numpy front end does). */
int ctr_bp_fan_2d_angle_prep(const ctr_fan_bp_angle_param* p, const double* angles,
                             double* xpos, double* ypos, double* sincostbl,
                             cudaStream_t stream);
int ctr_bp_fan_2d_angle_f32(const ctr_fan_bp_angle_param* p, const float* proj, float* img,
                            const double* xpos, const double* ypos, const double* sincostbl,
                            int batch, cudaStream_t stream);
int ctr_bp_fan_2d_angle_f64(const ctr_fan_bp_angle_param* p, const double* proj, double* img,
                            const double* xpos, const double* ypos, const double* sincostbl,
                            int batch, cudaStream_t stream);
int ctr_bp_fan_2d_angle_grad_f32(const ctr_fan_bp_angle_param* p, const float* img,
                                 float* grad, const double* xpos, const double* ypos,
                                 const double* sincostbl, int batch, cudaStream_t stream);
int ctr_bp_fan_2d_angle_grad_f64(const ctr_fan_bp_angle_param* p, const double* img,
                                 double* grad, const double* xpos, const double* ypos,
                                 const double* sincostbl, int batch, cudaStream_t stream);

/* ---- parallel-beam pixel-driven backprojection
 *      (reference include/bp_par_2d.h:153-224) ----
 * Tables (ParallelBackprojection2DPixDrivenPrep): xcos double[nx][na] = x cos t,
 * ysin double[ny][na] = y sin t; `buffer` is unused, as in the reference.
 * Forward scale is the signed orbit.  Grad is the exact adjoint of the
 * forward and takes the forward's tables (the reference's grad pair,
 * include/bp_par_2d.h:181-224, is not well defined and is replaced). */
int ctr_bp_par_2d_prep(const ctr_par_param* p, double* xcos, double* ysin, int* buffer,
                       cudaStream_t stream);
int ctr_bp_par_2d_f32(const ctr_par_param* p, const float* proj, float* img,
                      const double* xcos, const double* ysin, const int* buffer, int batch,
                      cudaStream_t stream);
int ctr_bp_par_2d_f64(const ctr_par_param* p, const double* proj, double* img,
                      const double* xcos, const double* ysin, const int* buffer, int batch,
                      cudaStream_t stream);
int ctr_bp_par_2d_grad_f32(const ctr_par_param* p, const float* img, float* grad,
                           const double* xcos, const double* ysin, int batch,
                           cudaStream_t stream);
int ctr_bp_par_2d_grad_f64(const ctr_par_param* p, const double* img, double* grad,
                           const double* xcos, const double* ysin, int batch,
                           cudaStream_t stream);

/* ---- FP32 backprojection plans (in the reference:
 *      ParallelBackprojection2DPixDriven<float>::calculate_on_gpu,
 *      include/bp_par_2d.h:170-185, and FanBackprojection2DPixDriven<float>::
 *      calculate_on_gpu, include/bp_fan_2d.h:175-190, with the per-call set-up
 *      done once) ----
 * A plan copies the prep tables (read on `stream`, which it synchronises; the
 * caller's tables may be freed afterwards), and keeps the stream-split
 * scratch and each (32 x 64 tile, view)'s channel window and position
 * constants, so a run allocates nothing and starts with the taps.  Forward
 * results equal ctr_bp_par_2d_f32 / ctr_bp_fan_2d_f32 bit for bit.  A plan serves one
 * stream at a time, on the device it was made on; after a failed run destroy
 * it. */
typedef struct ctr_bp_plan ctr_bp_plan;
int ctr_bp_par_2d_plan_create(const ctr_par_param* p, const double* xcos, const double* ysin,
                              int max_batch, ctr_bp_plan** plan, cudaStream_t stream);
int ctr_bp_fan_2d_plan_create(const ctr_fan_bp_param* p, const double* xpos, const double* ypos,
                              const double* sincostbl, int max_batch, ctr_bp_plan** plan,
                              cudaStream_t stream);
int ctr_bp_plan_run(ctr_bp_plan* plan, const float* proj, float* img, int batch,
                    cudaStream_t stream);
/* The exact adjoint (ctr_bp_par_2d_grad_f32 / ctr_bp_fan_2d_grad_f32, bit for
 * bit up to the order of its float atomics), img [ny][nx] -> grad [na][ns]. */
int ctr_bp_plan_run_grad(ctr_bp_plan* plan, const float* img, float* grad, int batch,
                         cudaStream_t stream);
int ctr_bp_plan_destroy(ctr_bp_plan* plan);

/* ---- parallel-beam single-view backprojection
 *      (reference include/bp_par_2d_sv.h:112-138) ----
 * proj [na][ns] -> img [ny][nx][na]: the interpolated value of every view,
 * 0 where the pixel projects off the detector.  Same tables as bp_par_2d. */
int ctr_bp_par_2d_sv_f32(const ctr_par_param* p, const float* proj, float* img,
                         const double* xcos, const double* ysin, const int* buffer, int batch,
                         cudaStream_t stream);
int ctr_bp_par_2d_sv_f64(const ctr_par_param* p, const double* proj, double* img,
                         const double* xcos, const double* ysin, const int* buffer, int batch,
                         cudaStream_t stream);

/* ---- parallel-beam ray-driven forward projection
 *      (reference include/fp_par_2d.h:209-278) ----
 * Prep (ParallelProjection2DRayDrivenPrepare): sincostbl double[na][2],
 * beginoffset double[na][ns][2], usex int[na].  Grad prep
 * (...RayDrivenGradPrep): weights double[na], pos double[na][nx][2],
 * usex int[na].  Requires nx == ny, as the reference op does. */
int ctr_fp_par_2d_prep(const ctr_par_param* p, double* sincostbl, double* beginoffset,
                       int* usex, cudaStream_t stream);
int ctr_fp_par_2d_f32(const ctr_par_param* p, const float* img, float* proj,
                      const double* sincostbl, const double* beginoffset, const int* usex,
                      int batch, cudaStream_t stream);
int ctr_fp_par_2d_f64(const ctr_par_param* p, const double* img, double* proj,
                      const double* sincostbl, const double* beginoffset, const int* usex,
                      int batch, cudaStream_t stream);
int ctr_fp_par_2d_grad_prep(const ctr_par_param* p, double* weights, double* pos, int* usex,
                            cudaStream_t stream);
int ctr_fp_par_2d_grad_f32(const ctr_par_param* p, const float* proj, float* img,
                           const double* weights, const double* pos, const int* usex,
                           int batch, cudaStream_t stream);
int ctr_fp_par_2d_grad_f64(const ctr_par_param* p, const double* proj, double* img,
                           const double* weights, const double* pos, const int* usex,
                           int batch, cudaStream_t stream);

/* ---- ray-driven FP32 projection with a per-geometry plan (no counterpart
 *      in the reference: ParallelProjection2DRayDriven<float>::calculate_on_gpu,
 *      include/fp_par_2d.h:227-244, with the per-call ray set-up done once) ----
 * ctr_fp_par_2d_plan_create builds, from the prep tables above (read on
 * `stream`, which it synchronises; the tables may be freed afterwards), every
 * ray's fixed-point start and step, exact sample range and class (as a model
 * line per view plus the rays that differ from it), the reference's decisions
 * for rays that end within a rounding of the image border, and a
 * transposed-image workspace for max_batch images.  A run then gives the same
 * results as ctr_fp_par_2d_f32 bit for bit with no allocation: one launch for
 * one image (the projector makes its own transposed copy; a cooperative
 * launch), two for a batch (transposed copy, projector); img must be 16-byte
 * aligned.  A plan serves one stream at a time, on the device it was made on. */
typedef struct ctr_fp_plan ctr_fp_plan;
int ctr_fp_par_2d_plan_create(const ctr_par_param* p, const double* sincostbl,
                              const double* beginoffset, const int* usex, int max_batch,
                              ctr_fp_plan** plan, cudaStream_t stream);
int ctr_fp_par_2d_plan_run(ctr_fp_plan* plan, const float* img, float* proj, int batch,
                           cudaStream_t stream);
int ctr_fp_par_2d_plan_destroy(ctr_fp_plan* plan);

/* ---- parallel-beam ray-casting forward projection
 *      (reference include/fp_par_2d.h:155-203, src/fp_par_2d.cc:18-145) ----
 * Prep (ParallelProjection2DRayCastingPrepare, its step_size argument):
 * sincostbl double[na][2], begins double[na][ns][2] (the ray's entry point on
 * the FoV circle of radius fov, in pixel indices), nsteps int[na][ns].
 * Forward (ParallelProjection2DRayCasting): samples every step_size pixels;
 * the reference has no gradient for this method. */
int ctr_fp_par_2d_cast_prep(const ctr_par_param* p, double step_size, double* sincostbl,
                            double* begins, int* nsteps, cudaStream_t stream);
int ctr_fp_par_2d_cast_f32(const ctr_par_param* p, double step_size, const float* img,
                           float* proj, const double* sincostbl, const double* begins,
                           const int* nsteps, int batch, cudaStream_t stream);
int ctr_fp_par_2d_cast_f64(const ctr_par_param* p, double step_size, const double* img,
                           double* proj, const double* sincostbl, const double* begins,
                           const int* nsteps, int batch, cudaStream_t stream);

/* ---- parallel-beam distance-driven forward projection and its gradient
 *      (reference include/fp_par_2d.h:283-352, src/fp_par_2d.cc:396-653) ----
 * Prep (ParallelProjection2DDisDrivenPrep): sincostbl double[na][2],
 * beginoffset double[na][ns][3] (footprint centre, step per line, half width),
 * usex int[na].  Grad prep (...DisDrivenGradPrep): weights double[na],
 * pos double[na][nx][2], usex int[na].  The grad is the reference's
 * (ParallelProjection2DDisDrivenGrad), which is not the adjoint of the
 * length-normalised forward.  Requires nx == ny, as the reference op does. */
int ctr_fp_par_2d_dd_prep(const ctr_par_param* p, double* sincostbl, double* beginoffset,
                          int* usex, cudaStream_t stream);
int ctr_fp_par_2d_dd_grad_prep(const ctr_par_param* p, double* weights, double* pos, int* usex,
                               cudaStream_t stream);
int ctr_fp_par_2d_dd_f32(const ctr_par_param* p, const float* img, float* proj,
                         const double* sincostbl, const double* beginoffset, const int* usex,
                         int batch, cudaStream_t stream);
int ctr_fp_par_2d_dd_f64(const ctr_par_param* p, const double* img, double* proj,
                         const double* sincostbl, const double* beginoffset, const int* usex,
                         int batch, cudaStream_t stream);
int ctr_fp_par_2d_dd_grad_f32(const ctr_par_param* p, const float* proj, float* img,
                              const double* weights, const double* pos, const int* usex,
                              int batch, cudaStream_t stream);
int ctr_fp_par_2d_dd_grad_f64(const ctr_par_param* p, const double* proj, double* img,
                              const double* weights, const double* pos, const int* usex,
                              int batch, cudaStream_t stream);

/* ---- allocation-free FP32 forward projection (no counterpart in the
 *      reference; same arguments and results as ctr_fp_par_2d_f32) ----
 * For callers that cannot allocate device memory inside a call: a host that
 * owns all device memory (its own pool or a fixed arena), or a real-time loop
 * that must not wait on the allocator.  The scratch the projector needs (a
 * transposed copy of the image and per-call ray tables) is a fixed 16 MiB
 * array inside the library, so this call
 * allocates nothing.  Limits: 24 bytes per ray (na * ns) plus 4 bytes per
 * image pixel of the batch plus about 400 KB within 16 MiB (720 views x 729
 * bins with up to 3 images of 512 x 512), nx at most 8192, img 16-byte
 * aligned; otherwise CTR_ERR_UNSUPPORTED.
 * Every call looks up the array's address in the current context
 * (cudaGetSymbolAddress: cheap once the library's module is loaded, and
 * never stale after a device reset); the first call in a context loads the
 * module, so make it before any stream capture.  All calls on a device share
 * the array: calls ordered on one stream are fine, calls that may overlap
 * (other streams, other host threads) race on it. */
int ctr_fp_par_2d_f32_noalloc(const ctr_par_param* p, const float* img, float* proj,
                              const double* sincostbl, const double* beginoffset,
                              const int* usex, int batch, cudaStream_t stream);


/* ---- batched uneven fan-beam FBP (no reference counterpart: the reference
 *      loops over batch items of one geometry, tensorflow/bp_fan_2d_ops.h:119-125) ----
 * A plan reconstructs n items, each with its own FanBackprojection2DParam:
 * fan weighting (type 1 fan / 2 flat) -> ramp filter (matching type) ->
 * bp_fan_2d, as one batched filter launch and ONE persistent backprojection
 * launch over all (item, tile) pairs, optionally captured in a CUDA graph and
 * autotuned (tile shape, view-block depth) on the batch at creation.  The plan
 * owns its tables and a filtered-sinogram workspace; run() takes HOST arrays
 * of n DEVICE pointers (sinogram [na][ns] and image [ny][nx] per item) and is
 * stream-ordered.  A plan serves one stream at a time. */
typedef struct ctr_fbp_plan ctr_fbp_plan;
typedef struct ctr_fbp_plan_info {
    int n_items;
    long long work_items;        /* (item, tile) pairs */
    int tile_rows;               /* tile is 32 x tile_rows pixels */
    int view_block;              /* views per group per staged block */
    int ctas;                    /* persistent CTAs */
    int autotuned;
    double tuned_ms;             /* autotuner's time of the chosen config */
    int graph;                   /* run() replays a CUDA graph */
    unsigned long long workspace_bytes;
    long long launches_per_run;  /* kernels (and memset) per run */
} ctr_fbp_plan_info;
#define CTR_PLAN_AUTOTUNE 1
#define CTR_PLAN_GRAPH 2
int ctr_fbp_fan_plan_create(const ctr_fan_bp_param* geoms, int n_items, int weighting, int flags,
                            ctr_fbp_plan** plan);
int ctr_fbp_fan_plan_run(ctr_fbp_plan* plan, const float* const* proj, float* const* img,
                         cudaStream_t stream);
int ctr_fbp_fan_plan_info(const ctr_fbp_plan* plan, ctr_fbp_plan_info* info);
int ctr_fbp_fan_plan_destroy(ctr_fbp_plan* plan);

/* ---- helical rebinning: HelicalInterpolation360<T> / HelicalInterpolation180<T>
 *      (reference include/helical_interpolation.h:17-116, src/helical_interpolation.cc:80-370;
 *      CPU-only there) ----
 * Input [na][nt][ns] (view, detector row, channel), output
 * [nz][view_per_rot][ns]: one fan-beam sinogram per slice z0 + iz*dz (dz added
 * iz times).  The result equals the reference's bit for bit (FP64 arithmetic
 * in its order for both T).  As in the reference, dt and orbit_start are
 * unused: slab edges map to detector rows as z * dsd / dso.
 *
 * ctr_helical_interpolation_prep fills a caller-owned device table of
 * ctr_helical_interpolation_table_bytes(p) bytes for one method (per-channel
 * cos(gamma) and complementary rays, per-slice view ranges).  The run entry
 * points OR bits into status[b*nz + iz], one device word per item and slice
 * (zero them first; read them after the stream).  The reference processes
 * slices in order and throws at the first problem; the first slice (in order)
 * with a nonzero word names it:
 *   CTR_HELICAL_NO_VIEWS  the slice needs views outside [0, na): the
 *                         reference's "View not enough for this slice!" (the
 *                         slice is not written);
 *   CTR_HELICAL_NO_ROWS   a sample has no detector row in either ray: "No row
 *                         data available!" (the sample is written as 0);
 *   CTR_HELICAL_OUTSIDE   (not an error) a 180LI complementary sample lies in a
 *                         view before view 0; the reference reads out of
 *                         bounds there, here it reads 0.  Only possible when a
 *                         slice's first view is 0;
 *   CTR_HELICAL_BAD_TABLE the table was prepared for another method or
 *                         geometry (nothing is written; reported in word 0). */
typedef struct ctr_helical_param {
    unsigned int ns, nt, na;
    double ds, dt, offset_s, offset_t, orbit_start, orbit, couch_begin, couch_mov;
    unsigned int view_per_rot, nz;
    double dz, z0, thickness, dso, dsd;
} ctr_helical_param;
#define CTR_HELICAL_360 0
#define CTR_HELICAL_180 1
#define CTR_HELICAL_NO_ROWS 1u
#define CTR_HELICAL_OUTSIDE 2u
#define CTR_HELICAL_BAD_TABLE 4u
#define CTR_HELICAL_NO_VIEWS 8u
size_t ctr_helical_interpolation_table_bytes(const ctr_helical_param* p);
int ctr_helical_interpolation_prep(const ctr_helical_param* p, int method, void* table,
                                   cudaStream_t stream);
int ctr_helical_interpolation_360_f32(const ctr_helical_param* p, const float* in, float* out,
                                      const void* table, unsigned int* status, int batch,
                                      cudaStream_t stream);
int ctr_helical_interpolation_360_f64(const ctr_helical_param* p, const double* in, double* out,
                                      const void* table, unsigned int* status, int batch,
                                      cudaStream_t stream);
int ctr_helical_interpolation_180_f32(const ctr_helical_param* p, const float* in, float* out,
                                      const void* table, unsigned int* status, int batch,
                                      cudaStream_t stream);
int ctr_helical_interpolation_180_f64(const ctr_helical_param* p, const double* in, double* out,
                                      const void* table, unsigned int* status, int batch,
                                      cudaStream_t stream);

/* ---- numpy extension ABI (reference numpy_ext, the *_npext.cu files and common.cu) ----
 * Same names and signatures as the reference's libnumpy_ctext: handles over
 * HOST double arrays, FP64 kernels, blocking.  set_device(-1) (the reference's
 * CPU mode) returns false: this library is the GPU implementation only.
 * Failures return false (or -1 from *_create) with ctr_last_error(). */
bool set_device(const int device);                                /* common.cu:29-49 */
bool clear(void);                                                 /* common.cu:51-60 */
int fan_weighting_create(unsigned int ns, unsigned int nrow, double ds, double offset,
                         double dso, double dsd, int type);       /* fan_weighting_npext.cu:86-93 */
bool fan_weighting_run(int handle, double* in, double* out);      /* :95-100 */
bool fan_weighting_destroy(int handle);                           /* :102-106 */
int ramp_filter_create(unsigned int ns, unsigned int nrow, double ds, double dsd,
                       int type);                                 /* filter_npext.cu:104-111 */
bool ramp_filter_run(int handle, double* in, double* out);        /* :113-118 */
bool ramp_filter_destroy(int handle);                             /* :120-124 */
int fan_bp_2d_angle_create(double* angles, unsigned int ns, unsigned int na, double ds,
                           double offset_s, unsigned int nx, unsigned int ny, double dx,
                           double dy, double offset_x, double offset_y, double dso, double dsd,
                           double fov);                           /* bp_fan_2d_angle_npext.cu:136-146 */
bool fan_bp_2d_angle_run(int handle, double* in, double* out);    /* :148-153 */
bool fan_bp_2d_angle_destroy(int handle);                         /* :155-159 */

#ifdef __cplusplus
}
#endif
#endif
