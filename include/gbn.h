/*
 * gbn.h - C ABI of the GB300 tTV-NESTA library (libgbnesta.so).
 *
 * This is the drop-in boundary for OpenCLIPER's compressed-sensing hot path:
 * the NESTA solver with temporal total variation over multicoil Cartesian
 * k-space (src/processes/nesta/NestaUp.cpp) and the operator processes it is
 * built from.  The reference exposes these as C++ Process classes with
 * init()/launch() on XData/KData/SensitivityMapsData objects; the C++ facade in
 * include/OpenCLIPER/ keeps that API and forwards to the functions below.
 *
 * Conventions
 *  - Complex data are interleaved complex64 (re, im float pairs), passed as
 *    float* whose element count is 2x the number of complex values.
 *  - Layouts are the reference's (Data.cpp:1305-1343, width fastest):
 *      XData              [F][H][W]
 *      KData              [F][C][H][W]
 *      SensitivityMaps    [C][H][W]
 *      pixel mask (uint8) [F][H][W], 0 = not sampled (SamplingMasksData PIXELMASK)
 *      row mask (uint32)  [F][H], 0/1 per phase-encode line (ROWMASK)
 *  - W (columns, readout) must be a multiple of 8 (Data.cpp:1360-1372).  FFT
 *    lengths W and H must be 7-smooth and in [8, 512] (clFFT radices 2,3,5,7).
 *  - Pointers named d_* are device pointers on the context's device; every
 *    call is asynchronous on the context stream unless documented otherwise.
 *  - Every function returns GBN_OK (0) or a negative GBN_ERR_* code;
 *    gbn_last_error_string() describes the last failure of the calling thread.
 *    The reference throws CLError/std::invalid_argument (Utils.hpp:67-83); the
 *    C++ facade turns these codes back into exceptions.
 *  - A context is used by one host thread at a time, like the reference's
 *    CLapp with its single in-order queue (src/Process.cpp:53-56).
 */
#ifndef GBN_H
#define GBN_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GBN_API __attribute__((visibility("default")))
#else
#define GBN_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GBN_VERSION 1

enum {
  GBN_OK = 0,
  GBN_ERR_INVALID = -1,     /* bad argument (reference: std::invalid_argument) */
  GBN_ERR_UNSUPPORTED = -2, /* size/shape outside what this library implements */
  GBN_ERR_CUDA = -3,        /* CUDA runtime failure (reference: CLError) */
  GBN_ERR_NOMEM = -4        /* device allocation failed */
};

/* TemporalTV::Direction (include/OpenCLIPER/processes/nesta/TemporalTV.hpp:47) */
enum { GBN_TTV_ADJOINT = 0, GBN_TTV_FORWARD = 1 };
/* FFT::Direction = clfftDirection (include/OpenCLIPER/processes/FFT.hpp:74-79) */
enum { GBN_FFT_FORWARD = -1, GBN_FFT_BACKWARD = 1 };
/* ComplexElementProd::ConjugateSensMap_t (ComplexElementProd.hpp:48-56) */
enum { GBN_NOT_CONJUGATE = 0, GBN_CONJUGATE = 1 };

typedef struct gbn_ctx gbn_ctx;
typedef struct gbn_problem gbn_problem;
typedef struct gbn_batch gbn_batch;

/* ------------------------------------------------------------------------ */
/* Runtime: replaces CLapp (src/CLapp.cpp:188-575: platform/device/context/  */
/* queue) and the device-buffer registry (CLapp::addData, CLapp.cpp:1735).   */
/* ------------------------------------------------------------------------ */
GBN_API const char* gbn_last_error_string(void);
GBN_API int gbn_version(void);
/* number of supported FFT lengths written to out (up to cap); returns count */
GBN_API int gbn_supported_lengths(int* out, int cap);

/* CLapp::create (CLapp.hpp:239-240): bind device `device`, create a stream. */
GBN_API int gbn_ctx_create(int device, gbn_ctx** out);
GBN_API int gbn_ctx_destroy(gbn_ctx* ctx);
/* the cudaStream_t every call of this context is issued on */
GBN_API int gbn_ctx_get_stream(gbn_ctx* ctx, void** stream);
/* issue on a caller-owned cudaStream_t instead (NULL restores the own stream) */
GBN_API int gbn_ctx_set_stream(gbn_ctx* ctx, void* stream);
/* CLapp::getCommandQueue().finish() */
GBN_API int gbn_ctx_sync(gbn_ctx* ctx);
/* State of the drand48 generator used by the power-method restart
 * (NestaUp.cpp:369-385).  A new context starts like a fresh process
 * (glibc's default state, as if seed48 were never called). */
GBN_API int gbn_ctx_seed48(gbn_ctx* ctx, const unsigned short seed16v[3]);
GBN_API int gbn_ctx_get_rand48(gbn_ctx* ctx, unsigned short state16v[3]);
/* tuning knobs: "row_local" (1, default: problems whose kept k-space rows are
 * each fully sampled or unsampled -- every phase-encode row mask -- run the
 * one-kernel row-local iteration; 0: always the three-pass iteration),
 * "k1_coils_per_block", "k2_ctas_per_sm" (>= 1),
 * "mixed_adjoint_tc" (0/1: the mixed form also runs the adjoint column pass on
 * the tensor cores) and "mixed_fwd_tc" (1: the mixed form's forward column
 * pass always on the tensor cores, 0: never -- its groups then run the plain
 * FP32 kernels --, -1 (default): per (W, H) group, as gbn_autotune measured
 * for the nearest tuned shape, else on the tensor cores when H >= 320); the
 * mixed knobs are read when a batch is created */
GBN_API int gbn_ctx_set_tuning(gbn_ctx* ctx, const char* key, int value);
/* number of kernels this context has launched so far */
GBN_API int gbn_ctx_launch_count(gbn_ctx* ctx, unsigned long long* count);

/* Kernel-group timing with CUDA events on the context stream, the analogue of
 * ProfileParameters{enable} and ProcessCore::getKernelGroupExecutionTimes
 * (ProcessCore.hpp:71-84, ProcessCore.cpp:270-300).  While enabled, every
 * launch of a group is bracketed by two events; gbn_ctx_profile_read waits for
 * the stream and returns the launches and summed milliseconds of one group. */
enum {
  GBN_PROF_FWD_COLS = 0, /* forward column pass (S x -> kept rows)        */
  GBN_PROF_ROWS = 1,     /* row pass (residual and its row transform)     */
  GBN_PROF_INV_COLS = 2, /* adjoint column pass + tTV gradient + update   */
  GBN_PROF_SETUP = 3,    /* x0, maxima, norm estimate, row analysis       */
  GBN_PROF_OUTER = 4,    /* continuation-loop begin/end copies            */
  GBN_PROF_ITER = 5,     /* row-local iteration: columns, residual, update */
  GBN_PROF_KINDS = 6
};
GBN_API int gbn_ctx_profile(gbn_ctx* ctx, int enable);
GBN_API int gbn_ctx_profile_read(gbn_ctx* ctx, int kind, unsigned long long* launches, double* total_ms);
GBN_API int gbn_ctx_profile_reset(gbn_ctx* ctx);

/* Device memory (DeviceDataProperties::createEmptyDeviceBuffers,
 * DeviceDataProperties.cpp:156-230; host2Device/device2Host 383-398). */
GBN_API int gbn_alloc(gbn_ctx* ctx, size_t bytes, void** d_ptr);
GBN_API int gbn_free(gbn_ctx* ctx, void* d_ptr);
GBN_API int gbn_upload(gbn_ctx* ctx, void* d_dst, const void* h_src, size_t bytes);
GBN_API int gbn_download(gbn_ctx* ctx, void* h_dst, const void* d_src, size_t bytes);
/* like gbn_download but returns without waiting (h_dst should be page-locked) */
GBN_API int gbn_download_async(gbn_ctx* ctx, void* h_dst, const void* d_src, size_t bytes);
/* Prefetch: host->device copies on the context's second (copy) stream, so
 * that the next reconstruction's inputs travel while the current one is
 * solved (the reference's asynchronous KData load, KData.cpp:281-284, feeding
 * the solver queue).  h_src should be pinned for the copy to overlap.
 * gbn_copy_wait_compute: copies enqueued after it wait for all work enqueued
 * on the compute stream so far (e.g. the last solve that read the buffer).
 * gbn_compute_wait_copy: work enqueued on the compute stream after it waits
 * for all copies enqueued so far.  Double buffering, per step k:
 *   gbn_compute_wait_copy; gbn_copy_wait_compute;
 *   gbn_copy_upload(inputs of k+1 -> buffer set (k+1)%2);
 *   gbn_nesta_run(problem on buffer set k%2); gbn_download_async(result k). */
GBN_API int gbn_copy_upload(gbn_ctx* ctx, void* d_dst, const void* h_src, size_t bytes);
GBN_API int gbn_copy_wait_compute(gbn_ctx* ctx);
GBN_API int gbn_compute_wait_copy(gbn_ctx* ctx);
GBN_API int gbn_memset(gbn_ctx* ctx, void* d_dst, int value, size_t bytes);
/* page-locked host buffers for fast transfers */
GBN_API int gbn_host_alloc(size_t bytes, void** h_ptr);
GBN_API int gbn_host_free(void* h_ptr);

/* ------------------------------------------------------------------------ */
/* Operators (one entry per Process on the NESTA path).                     */
/* ------------------------------------------------------------------------ */
/* TemporalTV (TemporalTV.cpp:49-86; temporalTV.cl:49-107).
 * FORWARD: out[f] = in[f] - in[(f-1) mod F]
 * ADJOINT: out[f] = in[(f+1) mod F] - in[f]   (= -D^T, as the reference) */
GBN_API int gbn_op_ttv(gbn_ctx* ctx, int direction, const float* d_in, float* d_out, int W, int H, int F);
/* VectorNormalization (VectorNormalization.cpp:56-87; vectorNormalization.cl:42-56):
 * out = in / max(mu, |in|), n complex elements; in place allowed. */
GBN_API int gbn_op_normalize(gbn_ctx* ctx, const float* d_in, float* d_out, size_t n, float mu);
/* ComplexElementProd (ComplexElementProd.cpp:64-131; complexElementProd.cl:42-76):
 * out[f][c] = in[f] * S[c] (in_has_coils = 0, XData input) or in[f][c] * S[c]
 * (in_has_coils = 1, KData input), S conjugated when conjugate = 1. */
GBN_API int gbn_op_sensmul(gbn_ctx* ctx, int conjugate, const float* d_in, int in_has_coils, const float* d_S, float* d_out,
                   int W, int H, int F, int C);
/* XImageSum (XImageSum.cpp:79-96; xImageSum.cl:42-61): out[f] = sum_c in[f][c] */
GBN_API int gbn_op_coilsum(gbn_ctx* ctx, const float* d_in, float* d_out, int W, int H, int F, int C);
/* ApplyMask (ApplyMask.cpp:21-51; applyMask.cl:5-40): data[f][c][p] = 0 where mask[f][p] == 0 */
GBN_API int gbn_op_mask(gbn_ctx* ctx, float* d_data, const uint8_t* d_mask, int W, int H, int F, int C);
/* SamplingMasksData::rowmask2pixelmask (SamplingMasksData.cpp:389-441): rows
 * with value 1 become 255, value 0 becomes 0; any other value is an error
 * (reported through the return code after a device round trip). */
GBN_API int gbn_op_rowmask_to_pixelmask(gbn_ctx* ctx, const uint32_t* d_rowmask, uint8_t* d_pixmask, int W, int H, int F);
/* ComplexAbs (complexAbs.cl:43-70): out = (|in|, 0); ComplexAbsPow2
 * (complexAbsPow2.cl:43-71): out = (|in|^2, 0).  n complex elements. */
GBN_API int gbn_op_abs(gbn_ctx* ctx, const float* d_in, float* d_out, size_t n);
GBN_API int gbn_op_abs2(gbn_ctx* ctx, const float* d_in, float* d_out, size_t n);
/* FFT process, dim = -1 (FFT.cpp:116-201, 456-542): 2-D C2C over (W, H) of
 * `batch` images stored back to back; FORWARD unscaled, BACKWARD scaled 1/(W*H);
 * no fftshift.  In place allowed. */
GBN_API int gbn_op_fft2(gbn_ctx* ctx, int direction, const float* d_in, float* d_out, int W, int H, int batch);
/* NestaUp::operatorA plus the 1/sqrt(N) post-scale (NestaUp.cpp:162-190, 712-718):
 * k[f][c] = mask[f] * FFT2(S[c] * x[f]) / sqrt(W*H) */
GBN_API int gbn_op_encode(gbn_ctx* ctx, const float* d_x, const float* d_S, const uint8_t* d_mask, float* d_k, int W, int H,
                  int F, int C);
/* NestaUp::operatorAt with the sqrt(N) pre-scale (NestaUp.cpp:117-151, 749-753):
 * x[f] = sum_c conj(S[c]) * IFFT2(sqrt(W*H) * k[f][c])   (no mask) */
GBN_API int gbn_op_encode_adjoint(gbn_ctx* ctx, const float* d_k, const float* d_S, float* d_x, int W, int H, int F, int C);

/* SimpleMRIRecon (src/processes/examples/SimpleMRIRecon.cpp:58-101):
 * x[f] = sum_c conj(S[c]) * IFFT2(y[f][c]).  The input is not modified. */
GBN_API int gbn_simple_recon(gbn_ctx* ctx, const float* d_y, const float* d_S, float* d_x, int W, int H, int F, int C);

/* RSoS (src/processes/RSoS.cpp:58-85, src/kernels/rss.cl:43-74):
 * x[f] = (sqrt(sum_c |k[f][c]|^2), 0) for KData k [F][C][H][W]. */
GBN_API int gbn_op_rss(gbn_ctx* ctx, const float* d_k, float* d_x, int W, int H, int F, int C);
/* SimpleMRIReconSOS (src/processes/examples/SimpleMRIReconSOS.cpp:54-118):
 * x[f] = RSoS(IFFT2(y[f][c])).  Unlike the reference, the input is not
 * transformed in place, and no .mat or timing files are written. */
GBN_API int gbn_simple_recon_sos(gbn_ctx* ctx, const float* d_y, float* d_x, int W, int H, int F, int C);

/* Allocation-free SimpleMRIRecon: same result as gbn_simple_recon, but no
 * device memory is allocated.  No counterpart in the reference.  For callers
 * that cannot call cudaMalloc (code running during CUDA-graph stream capture,
 * hosts that own all device memory in fixed pools): the working memory is a
 * fixed array inside the library (about 8.2 MiB per device, kept until the
 * process exits).  Limits: F*H*C*W <= 2^20 and F*H <= 8192, otherwise
 * GBN_ERR_UNSUPPORTED.  The first call on a device resolves the array's
 * device address; make that first call before any stream capture.  All calls
 * share the one array: calls that overlap on the GPU race, so serialise them. */
GBN_API int gbn_simple_recon_static(gbn_ctx* ctx, const float* d_y, const float* d_S, float* d_x, int W, int H,
                                    int F, int C);

/* ------------------------------------------------------------------------ */
/* NESTA (NestaUp::launch, NestaUp.cpp:442-910)                              */
/* ------------------------------------------------------------------------ */
/* NestaUp::LaunchParameters (NestaUp.hpp:67-83) without argsMC/showProgress
 * (motion compensation and display are not part of this library). */
typedef struct gbn_nesta_params {
  float lambda_i;
  float mu_f;
  float La;
  unsigned int maxIntIter;
  float tolVar;
  int verbose;
  unsigned int maxIter;
  unsigned int stoptest;
  unsigned int miniter;
} gbn_nesta_params;

typedef struct gbn_nesta_stats {
  float normU;        /* myNormest result (NestaUp.cpp:291-439) */
  float maxX, maxUX;  /* max|x0|, max|U x0| (NestaUp.cpp:521-568) */
  float lambda, muf, mu0;
  float mu_final;
  float tolVar_final; /* the reference writes this back into LaunchParameters::tolVar */
  float fx_final;     /* objective of the last inner iteration */
  float qp_final;
  int inner_iters;    /* inner iterations executed, all outer loops */
  int normest_iters;
  int kept_rows;      /* k-space rows carried by the solver (sampled or nonzero) */
  int status;         /* 0; nonzero when the device reported a failure of this run: 3 a tensor-core
                         wait ran out, 4 kept rows outgrew the mixed form's DFT operand, 5 a
                         motion-compensation mesh point outside the image, 6 kept rows beyond a
                         fitted row buffer were dropped */
} gbn_nesta_stats;

/* Binds the caller's device buffers (not copied, not modified):
 * y = KData [F][C][H][W], S = [C][H][W], mask = pixel mask [F][H][W].
 * Allocates the solver workspace. */
GBN_API int gbn_problem_create(gbn_ctx* ctx, int W, int H, int F, int C, const float* d_y, const float* d_S,
                       const uint8_t* d_mask, gbn_problem** out);
/* Refused while a live batch holds the problem (destroy the batch first). */
GBN_API int gbn_problem_destroy(gbn_problem* p);
/* The row pass keeps one buffer of k-space rows, by default as large as the
 * k-space (every row of every frame and coil), so that any later contents of
 * y and mask fit.  This analyses the current y and mask (waiting for the
 * stream) and resizes it to the rows they keep plus headroom_rows (at most
 * every row), which roughly halves a problem's device footprint at R >= 4.
 * A later run whose data keep more rows than that drops the excess and
 * reports gbn_nesta_stats::status = 6.  *kept_rows (may be NULL) receives the
 * rows kept now.  Call before the problem joins a batch. */
GBN_API int gbn_problem_fit_rows(gbn_problem* p, int headroom_rows, int* kept_rows);
/* MotionCompensation (direction GBN_TTV_FORWARD, MotionCompensation.cpp:57-78)
 * or AdjointMotionCompensation (GBN_TTV_ADJOINT, AdjointMotionCompensation.cpp:
 * 59-86) of XData [F][H][W]; meshes and bounding box as for
 * gbn_problem_set_motion.  Waits for completion; a mesh point interpolating
 * outside the image is an error. */
GBN_API int gbn_op_motion(gbn_ctx* ctx, int direction, const float* d_in, float* d_out, const float* d_xn,
                          const int* d_xmesh, const int bound_box[4], int W, int H, int F);
/* Motion-compensated sparsity operator for later runs of p (NestaUp with
 * argsMC, NestaUp.cpp:201-278; ArgumentsMotionCompensation,
 * GroupwiseRegistration.hpp:95-100): d_xn = deformed mesh [2][F][H][W] float,
 * d_xmesh = original mesh [2][W][H] int, both 1-based (not copied, kept
 * alive by the caller), bound_box = the 1-based bounding box (host, 4 ints).
 * As in the reference, such a run starts from the image already in its output
 * buffer instead of E^H y.  All three NULL switches motion compensation off.
 * Mesh points whose interpolation leaves the image are skipped and reported
 * in gbn_nesta_stats::status. */
GBN_API int gbn_problem_set_motion(gbn_problem* p, const float* d_xn, const int* d_xmesh, const int bound_box[4]);
/* ---- GroupwiseRegistration (motion estimation) ----------------------------
 * GroupwiseRegistration::InitParameters (GroupwiseRegistration.hpp:145-158);
 * the reference's defaults are tests/MRIRecon.cpp:121-129: W 1, flagW 1,
 * radius 40, E 3, Dp {4, 4}, nmax 100, et 0.01, eh 0.005,
 * lambda {0, 0.005, 0, 0.5}.  This library implements spline orders E = 1 to 3,
 * equal control spacing, and the circular region of interest (radius > 0);
 * the reference's whole-box mode (radius 0) stores a one-pixel bounding box
 * (GroupwiseRegistration.cpp:113-121) and is refused. */
typedef struct gbn_registration_params {
  float W;          /* weight of each displacement step (normalised by the ROI area) */
  int flagW;        /* adapt the weight: x1.2 after a decrease of the metric, /2 otherwise */
  int radius;       /* radius of the circular region of interest, pixels */
  int E;            /* spline order */
  int Dp[2];        /* control-point spacing, pixels */
  int nmax;         /* maximum gradient-descent iterations */
  float et;         /* displacement-norm threshold */
  float eh;         /* metric-variation threshold (fraction of the initial metric) */
  float lambda[4];  /* smoothness weights: 1st spatial, 2nd spatial, 1st temporal, 2nd temporal */
} gbn_registration_params;

/* Sizes the registration derives from (N, F, params) (init(),
 * GroupwiseRegistration.cpp:92-190): control points per side (the T arrays are
 * [2][F][cp][cp]), the 1-based bounding box of the region of interest
 * {first column, first row, last column, last row}, and its pixel count. */
typedef struct gbn_registration_info {
  int cp;
  int bound_box[4];
  int area;
} gbn_registration_info;

typedef struct gbn_registration_stats {
  int iterations;  /* gradient-descent iterations run */
  float H0;        /* metric of the unregistered frames */
  float H;         /* metric after the last iteration */
  float Wn;        /* final step weight */
  float Tdif;      /* norm of the last displacement update */
  int status;      /* 0, or 5: an interpolation corner left the image */
} gbn_registration_stats;

GBN_API int gbn_registration_info_get(int N, int F, const gbn_registration_params* params, gbn_registration_info* info);
/* GroupwiseRegistration::launch (GroupwiseRegistration.cpp:550-618): modulus
 * normalised to 500 (DataNormalization), then the gradient descent of
 * optimizer() (groupwiseRegistration/optimizer.cpp) on the B-spline control
 * displacements T.  d_images: [F][N][N] complex (the reconstruction to
 * register).  d_T_init: [2][F][cp][cp] starting displacements, or NULL for
 * zeros (the reference's TData on its first motion iteration); it may be d_T
 * itself.  Outputs, all
 * device: d_T [2][F][cp][cp], d_xn the deformed mesh [2][F][N][N] (1-based,
 * horizontal then vertical), d_xmesh the original mesh [2][N][N] (int,
 * 1-based, as ArgumentsMotionCompensation::xData); d_xn, d_xmesh and
 * info.bound_box are the inputs of gbn_problem_set_motion.  h_H (host, may be
 * NULL): the metric per iteration, params->nmax + 1 floats.  Waits for
 * completion. */
GBN_API int gbn_registration_run(gbn_ctx* ctx, const float* d_images, int N, int F,
                                 const gbn_registration_params* params, const float* d_T_init, float* d_T,
                                 float* d_xn, int* d_xmesh, float* h_H, gbn_registration_stats* stats);

/* One reconstruction into d_x ([F][H][W], the reference's output XData).
 * Runs asynchronously; when stats != NULL the call waits for completion and
 * fills *stats. */
GBN_API int gbn_nesta_run(gbn_ctx* ctx, gbn_problem* p, const gbn_nesta_params* params, float* d_x, gbn_nesta_stats* stats);
/* End-to-end form with host buffers: uploads y, S and the pixel mask, runs,
 * downloads x, and returns when x is on the host. */
GBN_API int gbn_nesta_run_host(gbn_ctx* ctx, int W, int H, int F, int C, const float* h_y, const float* h_S,
                       const uint8_t* h_mask, const gbn_nesta_params* params, float* h_x, gbn_nesta_stats* stats);

/* ------------------------------------------------------------------------ */
/* Batched form.  No reference counterpart: the reference runs one           */
/* NestaUp::launch at a time; a batch gives the same results as running its  */
/* problems one after another in batch order (power-method draws included).  */
/* ------------------------------------------------------------------------ */
#define GBN_PRECISION_FP32 0  /* complex64 data and arithmetic, as the reference */
#define GBN_PRECISION_MIXED 1 /* column transforms on the tensor cores (split fp16 operands, FP32 accumulation) */

/* Plans n reconstructions: problems[i] (from gbn_problem_create on ctx, each
 * at most once), params[i], output image d_outputs[i] ([F][H][W] complex).
 * Problems of equal (W, H) share the launches of every solver pass (up to 64
 * per group); groups run concurrently.  A problem must not be run elsewhere
 * while a launch of the batch is in flight. */
GBN_API int gbn_batch_create(gbn_ctx* ctx, int n, gbn_problem* const* problems, const gbn_nesta_params* params,
                             float* const* d_outputs, int precision_mode, gbn_batch** out);
/* Enqueues the whole batch on the context stream (asynchronous); replays the
 * captured graph when gbn_batch_capture was called. */
GBN_API int gbn_batch_launch(gbn_batch* b);
/* Captures the whole batch solve into one CUDA graph (nothing runs). */
GBN_API int gbn_batch_capture(gbn_batch* b);
/* Waits for the context stream, then fills *stats for problem i of the batch. */
GBN_API int gbn_batch_stats(gbn_batch* b, int i, gbn_nesta_stats* stats);
/* The batch's (W, H) groups of at most 64 members, and how many of them run
 * the forward column pass on the tensor cores (mixed form, "mixed_fwd_tc"). */
GBN_API int gbn_batch_groups(gbn_batch* b, int* groups, int* tensor_core_groups);
/* Group g (0 <= g < groups) of a batch: its W, H, member count, the members'
 * batch indices (member_idx: room for 64, or NULL) and the inner iteration it
 * runs (path: one of GBN_PATH_*).  No reference counterpart (the reference
 * solves one reconstruction per NestaUp::launch). */
#define GBN_PATH_THREE_PASS 0       /* forward column, row and adjoint column passes, FP32 */
#define GBN_PATH_THREE_PASS_TC 1    /* the same with the forward column pass on the tensor cores */
#define GBN_PATH_ROW_LOCAL 2        /* one fused kernel per iteration (row masks), FP32 */
#define GBN_PATH_ROW_LOCAL_TC 3     /* the row-local iteration on the tensor cores */
GBN_API int gbn_batch_group_info(gbn_batch* b, int g, int* W, int* H, int* members, int* member_idx, int* path);
GBN_API int gbn_batch_destroy(gbn_batch* b);
/* create + launch (+ stats for every problem when stats != NULL, which waits)
 * + destroy */
GBN_API int gbn_batch_run(gbn_ctx* ctx, int n, gbn_problem* const* problems, const gbn_nesta_params* params,
                          float* const* d_outputs, int precision_mode, gbn_nesta_stats* stats);
/* CUDA-graph names for the same operations: capture a batch, replay it. */
GBN_API int gbn_graph_capture(gbn_batch* b);
GBN_API int gbn_graph_replay(gbn_batch* b);

/* ------------------------------------------------------------------------ */
/* Launch-shape autotuner (no reference counterpart).                        */
/* ------------------------------------------------------------------------ */
/* For each shape (W, H, F, C) of `shapes` (n x 4 ints) times the run-time
 * launch shapes (coils per forward-column CTA, row-pass CTAs per SM) on a
 * synthetic problem and keeps the fastest in the context; later runs and
 * batches of that shape use it (the nearest tuned F, C of the same W, H
 * otherwise).  With a cache_path, shapes found in that text file are loaded
 * instead of measured and new results are appended.  The drand48 state is
 * left unchanged. */
GBN_API int gbn_autotune(gbn_ctx* ctx, int n, const int* shapes, const char* cache_path);
/* loads a cache file written by gbn_autotune */
GBN_API int gbn_autotune_load(gbn_ctx* ctx, const char* cache_path);
/* launch shapes a run of this shape would use */
GBN_API int gbn_autotune_lookup(gbn_ctx* ctx, int W, int H, int F, int C, int* k1_coils_per_block, int* k2_ctas_per_sm);

#ifdef __cplusplus
}
#endif

#endif /* GBN_H */
