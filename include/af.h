/*
 * af.h -- C ABI of libaf, the GB300 (sm_103a) implementation of the
 * accelerate-fourier transform hot path.
 *
 * The reference (accelerate-fourier 1.0.0.5, a Haskell/Accelerate library)
 * exposes its transforms as Accelerate functions
 *     type Transform sh a = Acc (Array sh a) -> Acc (Array sh a)
 * (src/Data/Array/Accelerate/Fourier/Private.hs:29).  A Haskell caller binds
 * the entry points below with `foreign import ccall` and wraps them in
 * Accelerate's foreign-function escape hatch; each entry point names the
 * reference function it replaces.
 *
 * Conventions (same as the reference):
 *   - arrays are row-major; the transform runs over the innermost axis, the
 *     leading axes are the batch ("sh" in `sh :. Int`);
 *   - sign -1 is `forward`, +1 is `inverse` (Fourier/Sign.hs:52-54), and no
 *     transform scales its result (use af_scale_down for Utility.scaleDown);
 *   - complex data is Complex Float32, either interleaved (re,im pairs) or
 *     planar (separate re and im arrays, Accelerate's own representation of
 *     `Array sh (Complex Float)`).
 * Library conventions:
 *   - every pointer is a device pointer owned by the caller; every call is
 *     asynchronous on the given CUDA stream and returns an af_status;
 *   - the library owns plans, twiddle tables and workspaces (released by
 *     af_plan_destroy);
 *   - a plan may be used from one stream at a time;
 *   - af_last_error() gives a readable message for the calling thread.
 */
#ifndef AF_H
#define AF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* af_stream; /* a cudaStream_t; NULL = legacy default stream */

typedef enum {
  AF_OK = 0,
  AF_ERR_INVALID = 1,     /* bad argument (size, sign, pointer, layout)      */
  AF_ERR_UNSUPPORTED = 2, /* valid request this build cannot run             */
  AF_ERR_CUDA = 3,        /* a CUDA runtime call failed                      */
  AF_ERR_ALLOC = 4,       /* device memory could not be allocated            */
  AF_ERR_TIMEOUT = 5      /* a bounded device-side wait gave up             */
} af_status;

/* Algorithm selection; each value names the reference function it mirrors. */
typedef enum {
  AF_ALGO_AUTO = 0,            /* Planned.transform          (Planned.hs:103-106) */
  AF_ALGO_DECOMPOSE = 1,       /* Planned.transformDecompose (Planned.hs:114-119) */
  AF_ALGO_CHIRP2 = 2,          /* Planned.transformChirp2    (Planned.hs:704-708) */
  AF_ALGO_CHIRP235 = 3,        /* Planned.transformChirp235  (Planned.hs:716-720) */
  AF_ALGO_PREP_DIT2 = 4,       /* Preprocessed.dit2          (Preprocessed.hs:99-111) */
  AF_ALGO_PREP_DIF2 = 5,       /* Preprocessed.dif2          (Preprocessed.hs:117-135) */
  AF_ALGO_PREP_SPLITRADIX = 6, /* Preprocessed.ditSplitRadix (Preprocessed.hs:53-93) */
  AF_ALGO_ADHOC_AUTO = 7,      /* Adhoc.transform            (Adhoc.hs:74-84)   */
  AF_ALGO_ADHOC_DIT2 = 8,      /* Adhoc.dit2                 (Adhoc.hs:138-153) */
  AF_ALGO_ADHOC_SPLITRADIX = 9,/* Adhoc.ditSplitRadix        (Adhoc.hs:101-108) */
  AF_ALGO_ADHOC_DIT235 = 10,   /* Adhoc.dit235               (Adhoc.hs:171-204) */
  AF_ALGO_ADHOC_CHIRP2 = 11,   /* Adhoc.transformChirp2      (Adhoc.hs:342-350) */
  AF_ALGO_ADHOC_CHIRP235 = 12  /* Adhoc.transformChirp235    (Adhoc.hs:355-362) */
} af_algo;

typedef enum { AF_LAYOUT_INTERLEAVED = 0, AF_LAYOUT_PLANAR = 1 } af_layout;

typedef struct af_plan_s* af_plan;

/* Library identification and the per-thread error message. */
const char* af_version(void);
const char* af_last_error(void);

/* Plans -------------------------------------------------------------------
 * Replaces Planned.plan/cache/transformWithCache (Planned.hs:137-167,201-203,
 * 322-328): af_plan_create runs the reference planner (bit-exact plan tree) and
 * builds the device twiddle tables in FP64, rounded to FP32.
 * Sizes must satisfy 0 <= n; the power-of-two and 5-smooth algorithms need
 * the sizes the reference functions accept (AF_ERR_INVALID otherwise). */
af_status af_plan_create(af_plan* plan, int64_t n, int sign, af_algo algo);
af_status af_plan_destroy(af_plan plan);
/* The reference plan tree as text, e.g. "GT1001(P13(SR12(SR6(S3))),...)". */
af_status af_plan_describe(af_plan plan, char* buf, size_t len);
/* The plan tree of Planned.plan for size n (no device work). */
af_status af_plan_tree(int64_t n, af_algo algo, char* buf, size_t len);
/* Number of kernel launches one af_exec_c2c with this batch issues. */
af_status af_plan_launches(af_plan plan, int64_t batch, int64_t* launches);

/* Complex-to-complex transform over `batch` rows of length n.
 * Replaces `transform sign len` / `transformWithCache` applied to an array of
 * shape (batch :. n) (Planned.hs:103-106,137-167) and the Preprocessed/Adhoc
 * transforms selected at plan time.
 * INTERLEAVED: in_re/out_re point at float2 data, in_im/out_im are NULL.
 * PLANAR: separate float arrays.  in == out (in place) is allowed. */
af_status af_exec_c2c(af_plan plan, af_layout layout, const float* in_re,
                      const float* in_im, float* out_re, float* out_im,
                      int64_t batch, af_stream stream);

/* Adjoint (VJP) of af_exec_c2c: grad = DFT^H(cot), i.e. the unscaled transform
 * of the opposite sign on the cotangent.  The reference has no AD; this is the
 * gradient of the transform with respect to its input. */
af_status af_vjp_c2c(af_plan plan, af_layout layout, const float* cot_re,
                     const float* cot_im, float* grad_re, float* grad_im,
                     int64_t batch, af_stream stream);

/* Complex Double ------------------------------------------------------------
 * The reference transforms are polymorphic over the element type
 * (`A.RealFloat a`, Planned.hs:103-106; Complex Double in its own tests,
 * test/Test/Data/Array/Accelerate/Fourier.hs:34-35).  af_plan_create_f64
 * builds a plan of the same reference tree whose tables, kernels and
 * workspaces hold Complex Double (FP64 throughout).  Such a plan runs only
 * through the _f64 entry points; the Complex Float entry points refuse it
 * (AF_ERR_INVALID), and the other way round.  af_plan_destroy,
 * af_plan_describe and af_plan_launches take either kind.
 * INTERLEAVED data is double2 (16-byte aligned); PLANAR is two double arrays. */
af_status af_plan_create_f64(af_plan* plan, int64_t n, int sign, af_algo algo);
af_status af_exec_c2c_f64(af_plan plan, af_layout layout, const double* in_re,
                          const double* in_im, double* out_re, double* out_im,
                          int64_t batch, af_stream stream);
/* Adjoint of af_exec_c2c_f64: grad = DFT^H(cot). */
af_status af_vjp_c2c_f64(af_plan plan, af_layout layout, const double* cot_re,
                         const double* cot_im, double* grad_re, double* grad_im,
                         int64_t batch, af_stream stream);

/* Utility.scaleDown (Fourier/Utility.hs:17-26): x *= 1/n over `batch` rows
 * of length n, in place. */
af_status af_scale_down(af_layout layout, float* re, float* im, int64_t n,
                        int64_t batch, af_stream stream);

/* Cyclic.reverse (Cyclic.hs:20-28): out[k] = in[(-k) mod n] per row.
 * in and out must not overlap. */
af_status af_cyclic_reverse(af_layout layout, const float* in_re,
                            const float* in_im, float* out_re, float* out_im,
                            int64_t n, int64_t batch, af_stream stream);

/* Cyclic.reverse2d (Cyclic.hs:30-39): out[y,x] = in[-y mod height,
 * -x mod width] for (batch, height, width) arrays; no overlap. */
af_status af_cyclic_reverse_2d(af_layout layout, const float* in_re,
                               const float* in_im, float* out_re, float* out_im,
                               int64_t height, int64_t width, int64_t batch,
                               af_stream stream);

/* Batches of mixed lengths ------------------------------------------------
 * `count` transforms of lengths lengths[0..count) stored back to back
 * (transform i starts at sum_{j<i} lengths[j]).  Each transform is planned
 * like Planned.transform (Planned.hs:103-106) computes it; every call is one
 * persistent launch whose CTAs take work items from a queue: whole transforms
 * of one CTA, and the stages of the two-pass four-step and three-pass
 * Bluestein schemes of longer ones (a stage's items start once the previous
 * stage's items have finished, through device counters with bounded waits;
 * the workspace stays in L2).  Batches with a Bluestein length above 131072,
 * or a 5-smooth length without a split into two factors of at most 1024,
 * run on a multi-launch plan instead.  Interleaved Complex Float32 only; one
 * call of a batch at a time.  The reference applies `transform` per array;
 * this entry point is the batched form of that call. */
typedef struct af_batch_s* af_batch;
af_status af_batch_create(af_batch* batch, const int64_t* lengths, int64_t count, int sign);
/* af_batch_create with the persistent executor's planner choices (stage
 * slack, lines per multi-pass item, radix-16 passes, item size) picked by
 * timing candidate plans of these lengths on the current device, on
 * `stream`; the choice is appended to the JSON-lines file `cache_path` (NULL:
 * no cache) under the GPU's name and a hash of the lengths, and reused from
 * there by later calls.  No counterpart in the reference, whose planner
 * (Planned.hs:206-214) picks algorithms by operation counts only. */
af_status af_batch_create_tuned(af_batch* batch, const int64_t* lengths, int64_t count, int sign,
                                const char* cache_path, af_stream stream);
/* JSON description of the batch: the executor, its work items, the planner
 * choices and the autotuner's report.  No counterpart in the reference. */
af_status af_batch_describe(af_batch batch, char* buf, size_t len);
af_status af_batch_destroy(af_batch batch);
af_status af_batch_launches(af_batch batch, int64_t* launches);
/* out = transform of every in (sign of the batch). */
af_status af_batch_exec(af_batch batch, const float* in, float* out, af_stream stream);
/* grad = DFT^H cot for every transform (the VJP of af_batch_exec). */
af_status af_batch_vjp(af_batch batch, const float* cot, float* grad, af_stream stream);
/* Waits for the batch's last call on `stream` and reports whether its
 * persistent launch completed: AF_ERR_TIMEOUT when a work item gave up its
 * bounded wait for the items of its previous stage (the outputs are then
 * incomplete).  No counterpart in the reference, whose transforms run to
 * completion inside `run`. */
af_status af_batch_status(af_batch batch, af_stream stream);
/* Forward transform with the spectral-weight epilogue of the loss
 * L = sum_i sum_k w_ik |X_ik|^2: writes cot = dL/dconj(X) * 2 = 2 w X and sets
 * *loss (device double) to L.  w holds one real weight per output element. */
af_status af_batch_forward_cotangent(af_batch batch, const float* x, const float* w, float* cot,
                                     double* loss, af_stream stream);

/* Multi-axis transforms -----------------------------------------------------
 * Along one axis of an (outer, n, inner) row-major array, n = plan's length,
 * with the plan's sign; inner = 1 is af_exec_c2c.  The reference transposes
 * (LinearAlgebra.transpose, Fourier/Private.hs:414-425 cycleDim3) around a
 * last-axis transform; here the kernels address the strided axis directly. */
af_status af_exec_c2c_axis(af_plan plan, af_layout layout, const float* in_re,
                           const float* in_im, float* out_re, float* out_im,
                           int64_t outer, int64_t inner, af_stream stream);
/* Adhoc.transform2d / Preprocessed.transform2d (Adhoc.hs:365-371,
 * Preprocessed.hs:142-149): an array (batch, n1, n0) with n0 = plan0's
 * length (last axis, the reference's least-significant `transform0`) and
 * n1 = plan1's length.  Each plan applies its own sign.  in == out allowed. */
af_status af_exec_c2c_2d(af_plan plan0, af_plan plan1, af_layout layout,
                         const float* in_re, const float* in_im, float* out_re,
                         float* out_im, int64_t batch, af_stream stream);
/* Adhoc.transform3d / Preprocessed.transform3d (Adhoc.hs:373-380,
 * Preprocessed.hs:151-160): (batch, n2, n1, n0), plan0 on the last axis. */
af_status af_exec_c2c_3d(af_plan plan0, af_plan plan1, af_plan plan2,
                         af_layout layout, const float* in_re,
                         const float* in_im, float* out_re, float* out_im,
                         int64_t batch, af_stream stream);
/* The same over Complex Double plans (af_plan_create_f64). */
af_status af_exec_c2c_2d_f64(af_plan plan0, af_plan plan1, af_layout layout,
                             const double* in_re, const double* in_im,
                             double* out_re, double* out_im, int64_t batch,
                             af_stream stream);
af_status af_exec_c2c_3d_f64(af_plan plan0, af_plan plan1, af_plan plan2,
                             af_layout layout, const double* in_re,
                             const double* in_im, double* out_re,
                             double* out_im, int64_t batch, af_stream stream);

/* Real transforms (Real.hs) ------------------------------------------------
 * `half` is the plan of the half-length complex transform the reference takes
 * as its `subTrans` argument: length N/2 for real rows of even length N. */
typedef enum {
  AF_SPECTRUM_FULL = 0, /* all N bins, as Real.toSpectrum returns them   */
  AF_SPECTRUM_HALF = 1  /* bins 0..N/2 (N/2+1 values), the rest is their
                           conjugate mirror; no reference counterpart   */
} af_spectrum;
/* Real.toSpectrum (Real.hs:49-70): x is batch x N reals (8-byte aligned),
 * out is batch x N (FULL) or batch x (N/2+1) (HALF) complex values. */
af_status af_to_spectrum(af_plan half, const float* x, af_spectrum spectrum,
                         af_layout layout, float* out_re, float* out_im,
                         int64_t batch, af_stream stream);
/* Real.fromSpectrum (Real.hs:92-108): a self-adjoint spectrum of N bins per
 * row -> N reals, unscaled; `half` is normally an inverse plan of N/2. */
af_status af_from_spectrum(af_plan half, af_layout layout, const float* spec_re,
                           const float* spec_im, float* x, int64_t batch,
                           af_stream stream);
/* Adjoint (VJP) of af_to_spectrum (FULL) with a forward `half` plan:
 * grad = Re(DFT_N^H cot) for a cotangent of N complex values per row, through
 * the half-length inverse transform.  The reference has no AD. */
af_status af_vjp_to_spectrum(af_plan half, af_layout layout, const float* cot_re,
                             const float* cot_im, float* grad, int64_t batch,
                             af_stream stream);

/* Two real signals through one complex transform (Real.hs:129-240).
 * twoToSpectrum: f, g are batch x n reals (the pair array's two components);
 * a, b receive their spectra.  The 2-D forms use af_exec_c2c_2d's shapes. */
af_status af_two_to_spectrum(af_plan plan, const float* f, const float* g,
                             af_layout layout, float* a_re, float* a_im,
                             float* b_re, float* b_im, int64_t batch,
                             af_stream stream);
af_status af_two_to_spectrum_2d(af_plan plan0, af_plan plan1, const float* f,
                                const float* g, af_layout layout, float* a_re,
                                float* a_im, float* b_re, float* b_im,
                                int64_t batch, af_stream stream);
/* twoFromSpectrum: entangle the two spectra, transform, and split the result
 * into its real (f) and imaginary (g) parts. */
af_status af_two_from_spectrum(af_plan plan, af_layout layout, const float* a_re,
                               const float* a_im, const float* b_re,
                               const float* b_im, float* f, float* g,
                               int64_t batch, af_stream stream);
af_status af_two_from_spectrum_2d(af_plan plan0, af_plan plan1, af_layout layout,
                                  const float* a_re, const float* a_im,
                                  const float* b_re, const float* b_im, float* f,
                                  float* g, int64_t batch, af_stream stream);
/* untangleSpectra (Real.hs:168-172): a = (s + conj(rev s))/2,
 * b = (s - conj(rev s))(-i/2).  s must not overlap a or b. */
af_status af_untangle_spectra(af_layout layout, const float* s_re,
                              const float* s_im, float* a_re, float* a_im,
                              float* b_re, float* b_im, int64_t n,
                              int64_t batch, af_stream stream);
/* untangleSpectra2d (Real.hs:174-179): the reverse runs over both axes of
 * (batch, height, width). */
af_status af_untangle_spectra_2d(af_layout layout, const float* s_re,
                                 const float* s_im, float* a_re, float* a_im,
                                 float* b_re, float* b_im, int64_t height,
                                 int64_t width, int64_t batch, af_stream stream);
/* entangleSpectra(2d) (Real.hs:207-236): out = c + i d, element-wise. */
af_status af_entangle_spectra(af_layout layout, const float* c_re,
                              const float* c_im, const float* d_re,
                              const float* d_im, float* out_re, float* out_im,
                              int64_t n, int64_t batch, af_stream stream);

/* Convolutions -------------------------------------------------------------
 * Planned.convolveCyclic (Planned.hs:779-821): out = F(G(x)/n * G(y)) with
 * G the inverse (+1) and F the forward (-1) transform of the plan's length
 * and algorithm (the plan's own sign is not used).  n must be non-zero. */
af_status af_convolve_cyclic(af_plan plan, af_layout layout, const float* x_re,
                             const float* x_im, const float* y_re,
                             const float* y_im, float* out_re, float* out_im,
                             int64_t batch, af_stream stream);
/* Convolution.Adhoc.karatsuba (Convolution/Adhoc.hs:36-98): linear
 * convolution of batch rows of length L into batch rows of 2L-1 (none for
 * L = 0).  Integer results are exact (two's-complement wrap-around, like the
 * reference's Int arithmetic); the i32 form widens its inputs to int64.
 * Floating-point results follow the reference's order of operations.
 * Scratch comes from the stream-ordered allocator (cudaMallocAsync). */
af_status af_karatsuba_i64(const int64_t* x, const int64_t* y, int64_t* z,
                           int64_t L, int64_t batch, af_stream stream);
af_status af_karatsuba_i32_i64(const int32_t* x, const int32_t* y, int64_t* z,
                               int64_t L, int64_t batch, af_stream stream);
af_status af_karatsuba_f32(const float* x, const float* y, float* z, int64_t L,
                           int64_t batch, af_stream stream);
af_status af_karatsuba_f64(const double* x, const double* y, double* z,
                           int64_t L, int64_t batch, af_stream stream);
/* Convolution.Adhoc.cyclic applied to a linear convolution z (batch x 2L-1,
 * Convolution/Adhoc.hs:104-111): out[k] = z[k] + z[k+L] (batch x L). */
af_status af_conv_cyclic_fold_i64(const int64_t* z, int64_t* out, int64_t L,
                                  int64_t batch, af_stream stream);
af_status af_conv_cyclic_fold_f32(const float* z, float* out, int64_t L,
                                  int64_t batch, af_stream stream);
af_status af_conv_cyclic_fold_f64(const double* z, double* out, int64_t L,
                                  int64_t batch, af_stream stream);
/* Convolution.Adhoc.complex (Convolution/Adhoc.hs:117-128) over karatsuba
 * (cyclic = 0: rows of 2L-1) or over `cyclic karatsuba` (cyclic = 1: rows of
 * L): three real convolutions (re*re, im*im, (re+im)*(re+im)).  Planar. */
af_status af_conv_complex_i64(int cyclic, const int64_t* x_re, const int64_t* x_im,
                              const int64_t* y_re, const int64_t* y_im,
                              int64_t* z_re, int64_t* z_im, int64_t L,
                              int64_t batch, af_stream stream);
af_status af_conv_complex_f32(int cyclic, const float* x_re, const float* x_im,
                              const float* y_re, const float* y_im, float* z_re,
                              float* z_im, int64_t L, int64_t batch,
                              af_stream stream);
af_status af_conv_complex_f64(int cyclic, const double* x_re, const double* x_im,
                              const double* y_re, const double* y_im,
                              double* z_re, double* z_im, int64_t L,
                              int64_t batch, af_stream stream);

/* Power-of-two transform that allocates no device memory.
 * This entry point has no counterpart in the reference.  It serves callers
 * that cannot call cudaMalloc: code running inside someone else's memory pool
 * or arena, work that must not touch the CUDA allocator while other work is
 * captured or timed, and embedders that forbid allocation after start-up.
 * It computes what af_exec_c2c computes for a power-of-two length n and
 * interleaved data, with its scratch workspace, twiddle tables and launch
 * descriptors in static device arrays of libaf (about 19 MiB, held by every
 * GPU that loads the library until the process exits).
 * Limit: n * batch <= 2^21 complex values; larger requests fail with
 * AF_ERR_INVALID and a message naming the limit.  The first call on a device
 * looks up the arrays' device addresses (once per device, with that device
 * current).  Calls cannot be captured in a CUDA graph: every call uploads its
 * launch descriptors from host memory, so a call on a capturing stream fails
 * with AF_ERR_UNSUPPORTED and leaves the capture untouched.  All calls share
 * the arrays and each call overwrites them, so calls that overlap on the GPU
 * race; calls issued to one stream are ordered. */
af_status af_exec_c2c_noalloc(int64_t n, int sign, const float* in, float* out,
                              int64_t batch, af_stream stream);

/* The Complex Double forms of the other entry points that carry complex or
 * real floating-point data, with the meaning, arguments and errors of the
 * Complex Float entry point of the same name without _f64.  The plan
 * arguments are Complex Double plans (af_plan_create_f64); the real arrays of
 * the real and two-real transforms are double. */
af_status af_exec_c2c_axis_f64(af_plan plan, af_layout layout,
                               const double* in_re, const double* in_im,
                               double* out_re, double* out_im, int64_t outer,
                               int64_t inner, af_stream stream);
af_status af_scale_down_f64(af_layout layout, double* re, double* im, int64_t n,
                            int64_t batch, af_stream stream);
af_status af_cyclic_reverse_f64(af_layout layout, const double* in_re,
                                const double* in_im, double* out_re,
                                double* out_im, int64_t n, int64_t batch,
                                af_stream stream);
af_status af_cyclic_reverse_2d_f64(af_layout layout, const double* in_re,
                                   const double* in_im, double* out_re,
                                   double* out_im, int64_t height,
                                   int64_t width, int64_t batch,
                                   af_stream stream);
af_status af_to_spectrum_f64(af_plan half, const double* x,
                             af_spectrum spectrum, af_layout layout,
                             double* out_re, double* out_im, int64_t batch,
                             af_stream stream);
af_status af_from_spectrum_f64(af_plan half, af_layout layout,
                               const double* spec_re, const double* spec_im,
                               double* x, int64_t batch, af_stream stream);
af_status af_vjp_to_spectrum_f64(af_plan half, af_layout layout,
                                 const double* cot_re, const double* cot_im,
                                 double* grad, int64_t batch, af_stream stream);
af_status af_untangle_spectra_f64(af_layout layout, const double* s_re,
                                  const double* s_im, double* a_re,
                                  double* a_im, double* b_re, double* b_im,
                                  int64_t n, int64_t batch, af_stream stream);
af_status af_untangle_spectra_2d_f64(af_layout layout, const double* s_re,
                                     const double* s_im, double* a_re,
                                     double* a_im, double* b_re, double* b_im,
                                     int64_t height, int64_t width,
                                     int64_t batch, af_stream stream);
af_status af_entangle_spectra_f64(af_layout layout, const double* c_re,
                                  const double* c_im, const double* d_re,
                                  const double* d_im, double* out_re,
                                  double* out_im, int64_t n, int64_t batch,
                                  af_stream stream);
af_status af_two_to_spectrum_f64(af_plan plan, const double* f, const double* g,
                                 af_layout layout, double* a_re, double* a_im,
                                 double* b_re, double* b_im, int64_t batch,
                                 af_stream stream);
af_status af_two_to_spectrum_2d_f64(af_plan plan0, af_plan plan1,
                                    const double* f, const double* g,
                                    af_layout layout, double* a_re,
                                    double* a_im, double* b_re, double* b_im,
                                    int64_t batch, af_stream stream);
af_status af_two_from_spectrum_f64(af_plan plan, af_layout layout,
                                   const double* a_re, const double* a_im,
                                   const double* b_re, const double* b_im,
                                   double* f, double* g, int64_t batch,
                                   af_stream stream);
af_status af_two_from_spectrum_2d_f64(af_plan plan0, af_plan plan1,
                                      af_layout layout, const double* a_re,
                                      const double* a_im, const double* b_re,
                                      const double* b_im, double* f, double* g,
                                      int64_t batch, af_stream stream);
af_status af_convolve_cyclic_f64(af_plan plan, af_layout layout,
                                 const double* x_re, const double* x_im,
                                 const double* y_re, const double* y_im,
                                 double* out_re, double* out_im, int64_t batch,
                                 af_stream stream);

#ifdef __cplusplus
}
#endif
#endif
