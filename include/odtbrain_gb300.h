/*
 * odtbrain_gb300 -- C ABI of the GB300 (sm_103a) 3D filtered backpropagation.
 *
 * The library replaces the compute of the reference's 3D backpropagation:
 *
 *   odtbrain.backpropagate_3d         odtbrain/_alg3d_bpp.py:84-555
 *   odtbrain.backpropagate_3d_tilted  odtbrain/_alg3d_bppt.py:374-949
 *
 * (also backpropagate_2d through a ny = 1 plan), and of the steps either
 * side of it, declared further down: odt_to_ri / opt_to_ri, the sinogram
 * preparation sinogram_as_rytov / sinogram_as_radon, and the
 * missing-apple-core correction apple.correct with its helpers
 * constraint_nn / constraint_sh / envelope_gauss.
 *
 * The reference is pure Python (NumPy + pyFFTW + numexpr + scipy.ndimage +
 * multiprocessing); it has no foreign-function interface of its own.  The
 * entry points below are what a binding of that Python path binds: the host
 * computes the FP64 constants exactly as the reference does (angle weights,
 * filter, propagator phase, rotation matrices and offsets) and hands plain
 * pointers to this library, which runs the per-angle pipeline on the GPU:
 *
 *   (a) pad + weight + forward 2D FFT + filter    _alg3d_bpp.py:493-509
 *   (b) per-plane propagator + inverse FFT + crop _alg3d_bpp.py:514-528
 *   (c) spline rotation + accumulation            _alg3d_bpp.py:532-546,
 *                                                 _alg3d_bppt.py:904-944
 *
 * All functions return an odt_status; none of them throws.  Device pointers
 * are raw CUDA device addresses; `stream` is a cudaStream_t passed as void*.
 * Execution is stream-ordered and does not synchronise the host, except
 * where a declaration says it is synchronous (the read_status calls, the
 * apple correction and envelope, the "sh" constraint).
 */
#ifndef ODTBRAIN_GB300_H
#define ODTBRAIN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum odt_status {
    ODT_OK = 0,
    ODT_ERR_INVALID_ARGUMENT = 1, /* maps to ValueError on the Python side   */
    ODT_ERR_UNSUPPORTED = 2,      /* maps to NotImplementedError             */
    ODT_ERR_CUDA = 3,             /* a CUDA runtime call failed              */
    ODT_ERR_OUT_OF_MEMORY = 4,    /* plan tables could not be allocated      */
    ODT_ERR_DEVICE_CHECK = 5      /* a kernel's own bounds check tripped     */
} odt_status;

enum odt_pad_mode {
    ODT_PAD_NONE = 0,  /* padding=(False, False)                 */
    ODT_PAD_EDGE = 1,  /* padval="edge": np.pad(mode="edge")     */
    ODT_PAD_RAMP = 2   /* padval=float: np.pad(mode="linear_ramp") */
};

enum odt_geometry {
    /* scipy.ndimage.rotate of every (z, x) plane about the y axis,
     * _alg3d_bpp.py:68-81; 6 doubles per angle: m00 m01 m10 m11 off0 off1 */
    ODT_GEOM_Y_AXIS = 0,
    /* scipy.ndimage.affine_transform of the (x, -y, z) volume,
     * _alg3d_bppt.py:904-944; 12 doubles per angle: 3x3 matrix row-major,
     * then the offset */
    ODT_GEOM_AFFINE3D = 1
};

enum odt_input_dtype { ODT_INPUT_C64 = 0, ODT_INPUT_C128 = 1 };

typedef struct odt_bpp3d_desc {
    int32_t num_angles;          /* A                                        */
    int32_t ny, nx;              /* sinogram plane; volume is (nx, ny, nx)  */
    int32_t pad_ny, pad_nx;      /* padded FFT sizes lNy, lNx               */
    int32_t pad_y_left;          /* padyl, _alg3d_bpp.py:300                */
    int32_t pad_x_left;          /* padxl, _alg3d_bpp.py:302                */
    int32_t pad_mode;            /* enum odt_pad_mode                       */
    double padval_re, padval_im; /* linear-ramp end value                   */
    int32_t intp_order;          /* spline order 0..5 (4, 5: nx >= 4, and  */
                                 /* ny >= 4 or 1 for AFFINE3D)              */
    int32_t geometry;            /* enum odt_geometry                       */
    int32_t onlyreal;            /* output float32 real part only           */
    int32_t input_dtype;         /* enum odt_input_dtype                    */
    /* Host arrays of pad_ny*pad_nx entries, row-major [ky][kx] in FFT order:
     * filter: complex128 (interleaved re, im) =
     *   prefactor [* filterabs] / (lNx*lNy)      _alg3d_bpp.py:389-399, 509
     * kz_phase: km*(M-1), the propagator phase per unit z  :419-437 */
    const double *filter;
    const double *kz_phase;
    uint64_t workspace_limit;    /* bytes of scratch the plan may use; 0 =
                                    library default (16 GiB)                */
    /* Position of plane p along the propagation axis: z_p = p - nz/2 +
     * z_shift.  0 for the 3D functions (_alg3d_bpp.py:419-437); 0.5 for the
     * 2D algorithm run as ny = 1 (rows yv = k - ln/2 + 0.5,
     * _alg2d_bpp.py:295-300). */
    double z_shift;
} odt_bpp3d_desc;

typedef struct odt_bpp3d_plan odt_bpp3d_plan;

/* Build a plan (device tables for the filter, the propagator and the FFT
 * twiddles).  Replaces the per-call setup of _alg3d_bpp.py:237-487.
 * ODT_ERR_UNSUPPORTED for FFT lengths other than powers of two in
 * [64, 4096] or lengths <= 1024, for spline orders 4 and 5 on lines of
 * fewer than 4 samples, and when one angle's coefficient slab
 * (nx * nx * ny rounded up to 32) would hold 2^31 elements or more. */
odt_status odt_bpp3d_plan_create(const odt_bpp3d_desc *desc,
                                 odt_bpp3d_plan **plan);

/* Bytes of device scratch odt_bpp3d_execute needs. */
odt_status odt_bpp3d_workspace_size(const odt_bpp3d_plan *plan,
                                    uint64_t *bytes);

/* Number of angles the plan processes per pass of the rotation kernel. */
odt_status odt_bpp3d_angle_batch(const odt_bpp3d_plan *plan, int32_t *batch);

/* Every call that takes a plan must be made with the device the plan was
 * created on current (cudaSetDevice); otherwise it returns
 * ODT_ERR_INVALID_ARGUMENT.
 *
 * Run the backpropagation (the loop of _alg3d_bpp.py:492-549).
 *   sino      device, (A, ny, nx) complex64 or complex128 (desc.input_dtype)
 *   weights   device, A doubles (angle weights, util.py:4-67) or NULL
 *   geometry  device, A*6 (Y_AXIS) or A*12 (AFFINE3D) doubles
 *   volume    device, (nx, ny, nx) complex64, or float32 when onlyreal;
 *             fully overwritten
 *   workspace device, odt_bpp3d_workspace_size bytes, 256-byte aligned
 * The row stage runs on a second stream that the plan owns, forked from and
 * joined back into `stream` with events (so the call also works inside
 * stream capture); a plan must not be executed by two host threads at
 * once. */
odt_status odt_bpp3d_execute(const odt_bpp3d_plan *plan, const void *sino,
                             const double *weights, const double *geometry,
                             void *volume, void *workspace, void *stream);

/* odt_bpp3d_execute with gains multiplying the filter, both in the
 * filter's [ky][kx] FFT order (NULL: none):
 *   gain        device, pad_ny*pad_nx floats, shared by all angles
 *   angle_gain  device, A*pad_ny*pad_nx complex64, one map per angle (the
 *               learned filter's output)
 * The gains are the learnable inputs of the differentiable reconstruction;
 * no counterpart in the reference. */
odt_status odt_bpp3d_execute_gain(const odt_bpp3d_plan *plan, const void *sino,
                                  const double *weights,
                                  const double *geometry, const float *gain,
                                  const void *angle_gain, void *volume,
                                  void *workspace, void *stream);

/* Bytes of device workspace odt_bpp3d_adjoint needs. */
odt_status odt_bpp3d_adjoint_workspace_size(const odt_bpp3d_plan *plan,
                                            uint64_t *bytes);

/* Vector-Jacobian product of odt_bpp3d_execute_gain (either geometry,
 * spline orders 0..3, complex output).  Given the volume cotangent vol_grad (nx, ny, nx)
 * complex64, writes (each may be NULL)
 *   sino_grad       (A, ny, nx) complex64 = J_sino^H vol_grad
 *   gain_grad       pad_ny*pad_nx float   = Re(J_gain^H vol_grad)
 *   angle_gain_grad A*pad_ny*pad_nx complex64 = J_angle_gain^H vol_grad
 * The gain gradients need `sino`.  The transpose of every stage is
 * computed, not stored: the spectra are recomputed from `sino` when a gain
 * gradient is asked for.  No counterpart in the reference (which has no
 * derivatives). */
odt_status odt_bpp3d_adjoint(const odt_bpp3d_plan *plan, const void *sino,
                             const double *weights, const double *geometry,
                             const float *gain, const void *angle_gain,
                             const void *vol_grad, void *sino_grad,
                             float *gain_grad, void *angle_gain_grad,
                             void *workspace, void *stream);

/* Per-stage record of one execution, for measurement. */
enum odt_stage {
    ODT_STAGE_ROWS_FORWARD = 0,      /* (a) pad, weight, forward FFT along x */
    ODT_STAGE_COLUMNS_PROPAGATE = 1, /* (b) FFT along y, filter, propagator,
                                        backward FFT along y               */
    ODT_STAGE_ROWS_INVERSE = 2,      /* (b) backward FFT along x, crop      */
    ODT_STAGE_ROTATE = 3,            /* (c) spline resampling + accumulation */
    ODT_NUM_STAGES = 4
};
typedef struct odt_stage_timing {
    double ms[ODT_NUM_STAGES];        /* summed CUDA-event time per stage */
    int64_t launches[ODT_NUM_STAGES]; /* kernel launches per stage        */
    double bytes[ODT_NUM_STAGES];     /* algorithmic HBM bytes per stage:
                                         (a) sinogram read + spectrum write,
                                         (b) spectrum read / slab write,
                                         (c) slab read + volume write      */
} odt_stage_timing;

/* odt_bpp3d_execute with a CUDA event pair around every kernel launch;
 * waits for `stream` and fills `timing`.  No counterpart in the reference
 * (measurement only). */
odt_status odt_bpp3d_execute_timed(const odt_bpp3d_plan *plan,
                                   const void *sino, const double *weights,
                                   const double *geometry, void *volume,
                                   void *workspace, void *stream,
                                   odt_stage_timing *timing);

/* Number of kernel launches one odt_bpp3d_execute makes. */
odt_status odt_bpp3d_launch_count(const odt_bpp3d_plan *plan,
                                  int64_t *launches);

/* Bytes of the library's static device scratch used by
 * odt_bpp3d_execute_noalloc. */
#define ODT_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* odt_bpp3d_execute without a workspace argument and without allocating:
 * for callers that cannot allocate device memory when they reconstruct (a
 * cudaMalloc there would synchronise the device, is forbidden while a stream
 * is captured, or the application's allocator owns all device memory).  The
 * scratch is a 64 MiB array in the library's device image, held by every
 * device that loads the library's device code until the process exits.
 * Plans whose workspace exceeds ODT_NOALLOC_SCRATCH_BYTES are rejected
 * (ODT_ERR_INVALID_ARGUMENT): create them with desc.workspace_limit <=
 * ODT_NOALLOC_SCRATCH_BYTES.  The first call on a device looks the array's
 * address up (make that call before any stream capture); all calls on a
 * device share the array, so calls whose executions overlap on the GPU race.
 * No counterpart in the reference. */
odt_status odt_bpp3d_execute_noalloc(const odt_bpp3d_plan *plan,
                                     const void *sino, const double *weights,
                                     const double *geometry, void *volume,
                                     void *stream);

/* ---- Learned filter gain ------------------------------------------------
 * A 4-layer MLP (4 -> 64 -> 64 -> 64 -> 2, SiLU, BF16 operands, FP32
 * accumulation on the tensor cores) that maps, for every angle a and padded
 * spectrum position (ky, kx), the features (2*kx/pad_nx, 2*ky/pad_ny in
 * fftfreq order, angle_features[2a], angle_features[2a+1]) to the complex
 * gain 1 + out_re + i*out_im, the angle_gain of odt_bpp3d_execute_gain.
 * No counterpart in the reference (its filter is fixed). */
typedef struct odt_mlp_params {
    const void *w1;   /* bf16 [64][16]: layer 1, columns 4..15 zero         */
    const void *w2;   /* bf16 [64][64]                                       */
    const void *w3;   /* bf16 [64][64]                                       */
    const void *w4;   /* bf16 [8][64]: rows 2..7 zero                        */
    const void *w2t;  /* bf16 [64][64]: transpose of w2 (training only)      */
    const void *w3t;  /* bf16 [64][64]: transpose of w3 (training only)      */
    const void *w4t;  /* bf16 [64][16]: transpose of w4, columns 8..15 zero  */
    const float *b1, *b2, *b3;  /* [64]                                      */
    const float *b4;            /* [8]: entries 2..7 zero                     */
} odt_mlp_params;             /* all pointers device, 16-byte aligned        */

typedef struct odt_mlp_grads {  /* FP32, the weights' shapes; added to (+=)  */
    float *w1, *w2, *w3, *w4;
    float *b1, *b2, *b3, *b4;   /* rows / entries of padding stay untouched  */
} odt_mlp_grads;

/* gain: complex64 [num_angles][pad_ny][pad_nx]; angle_features: float
 * [num_angles][2].  positions (device, optional): the num_positions flat
 * spectrum positions ky*pad_nx + kx evaluated for every angle, e.g. the
 * support of the filter; other gain entries are left untouched (NULL: all
 * pad_ny*pad_nx positions).  Listed positions outside the grid are skipped. */
odt_status odt_mlp_gain_forward(const odt_mlp_params *params,
                                int32_t num_angles, int32_t pad_ny,
                                int32_t pad_nx, const float *angle_features,
                                const int32_t *positions,
                                int32_t num_positions, void *gain,
                                void *stream);

/* Inference runs on the 5th-generation tensor cores (tcgen05.mma with the
 * accumulators in tensor memory), whose completion waits are bounded; wait
 * for `stream` and return ODT_ERR_DEVICE_CHECK if such a wait gave up since
 * the last call (the gains of that call are then invalid). */
odt_status odt_mlp_read_status(void *stream);

/* Kernel family of odt_mlp_gain_forward and odt_mlp_gain_backward, process
 * wide: 1 (the default) the tcgen05 kernels (BF16 operands, FP32
 * accumulators in tensor memory), 0 the same network on warp-level
 * mma.sync; both give the same results within BF16 rounding.  For
 * comparisons.  No counterpart in the reference. */
odt_status odt_mlp_select_kernels(int32_t tensor_memory);

/* Device bytes of the activation store odt_mlp_gain_backward needs for
 * num_positions positions per angle. */
odt_status odt_mlp_store_size(int32_t num_angles, int32_t num_positions,
                              uint64_t *bytes);

/* Gradients of a real loss with respect to the MLP parameters, given the
 * loss gradient with respect to the gain (complex64, PyTorch's convention
 * d/dRe + i d/dIm, e.g. the angle_gain_grad of odt_bpp3d_adjoint).  Recomputes
 * the forward; `store` (256-byte aligned, odt_mlp_store_size bytes) holds the
 * activations between the two kernels.  Only the listed positions
 * contribute (the gradient elsewhere must be zero for the result to be the
 * full gradient, as it is outside the filter's support). */
odt_status odt_mlp_gain_backward(const odt_mlp_params *params,
                                 int32_t num_angles, int32_t pad_ny,
                                 int32_t pad_nx, const float *angle_features,
                                 const int32_t *positions,
                                 int32_t num_positions,
                                 const void *gain_grad, void *store,
                                 const odt_mlp_grads *grads, void *stream);

/* ---- Object function -> refractive index --------------------------------
 * Elementwise, stream-ordered, `n` elements of `dtype` at device `f` into
 * device `ri` (same type; may alias).  FP32 for F32/C64, FP64 for F64/C128.
 *   odt_odt_to_ri: ri = nm * sqrt(f / km^2 + 1), km = 2 pi nm / res;
 *     principal root with non-negative real part for complex data, NaN
 *     where f / km^2 + 1 < 0 for real data.  Replaces odtbrain.odt_to_ri
 *     (odtbrain/_translate_ri.py:5-57).
 *   odt_opt_to_ri: ri = nm + f / (2 pi) * res.  Replaces odtbrain.opt_to_ri
 *     (odtbrain/_translate_ri.py:60-93). */
enum odt_data_type {
    ODT_DATA_F32 = 0, ODT_DATA_F64 = 1, ODT_DATA_C64 = 2, ODT_DATA_C128 = 3
};
odt_status odt_odt_to_ri(const void *f, void *ri, int64_t n, int32_t dtype,
                         double res, double nm, void *stream);
odt_status odt_opt_to_ri(const void *f, void *ri, int64_t n, int32_t dtype,
                         double res, double nm, void *stream);

/* ---- Sinogram preparation ------------------------------------------------
 * Replaces odtbrain.sinogram_as_rytov (odtbrain/_prepare_sino.py:105-182)
 * and odtbrain.sinogram_as_radon (odtbrain/_prepare_sino.py:60-102),
 * including align_unwrapped (odtbrain/_prepare_sino.py:7-46).
 * The sinogram is (A, nx) (ny = 0, numpy.unwrap along each line) or
 * (A, ny, nx) (ny > 0, reliability-sorted 2D unwrapping of every frame, the
 * algorithm of skimage.restoration.unwrap_phase that the reference calls).
 * The arithmetic type follows dtype: FP32 for complex64, FP64 for
 * complex128.  Output (device): RYTOV complex of dtype,
 * u0 * (log|u/u0| + 1j * unwrapped angle(u/u0)); RADON real (float32 /
 * float64), the unwrapped angle(u).  u0 (RYTOV only): the scalar
 * (u0_re, u0_im) when u0 == NULL, else a device array of dtype and the
 * sinogram's shape.  seed: seed of the pseudo-random border reliabilities
 * of the 3D unwrapping (the reference passes 47).
 * ODT_SINO_ALIGN: align_unwrapped alone; the input is a real unwrapped
 * phase sinogram (dtype ODT_DATA_F32 / F64, align = 1), the output its
 * aligned copy (may alias the input).
 * ODT_SINO_UNWRAP: the unwrapping alone (then alignment if `align`); the
 * input is a real wrapped phase (F32 / F64) of lines (ny = 0) or frames,
 * the output the unwrapped phase (may alias the input); for frames the
 * counterpart of skimage.restoration.unwrap_phase on each 2D frame.
 * Stream-ordered; the workspace (odt_sino_workspace_size bytes, 256-byte
 * aligned) also holds the status word that odt_sino_read_status reads. */
enum odt_sino_kind {
    ODT_SINO_RYTOV = 0, ODT_SINO_RADON = 1, ODT_SINO_ALIGN = 2, ODT_SINO_UNWRAP = 3
};
typedef struct odt_sino_desc {
    int64_t num_angles; /* A >= 1                                          */
    int32_t ny;         /* frame rows (3D sinogram), 0 for a 2D sinogram   */
    int32_t nx;         /* detector columns >= 1                           */
    int32_t dtype;      /* ODT_DATA_C64 or ODT_DATA_C128                   */
    int32_t kind;       /* odt_sino_kind                                   */
    int32_t align;      /* apply align_unwrapped                           */
    uint32_t seed;
    const void *u0;
    double u0_re, u0_im;
} odt_sino_desc;
odt_status odt_sino_workspace_size(const odt_sino_desc *desc, size_t *bytes);
odt_status odt_sino_prepare(const odt_sino_desc *desc, const void *sino,
                            void *out, void *workspace,
                            size_t workspace_bytes, void *stream);
/* Kernel launches one odt_sino_prepare call makes. */
odt_status odt_sino_launch_count(const odt_sino_desc *desc, int32_t *count);
/* Wait for `stream`; ODT_ERR_DEVICE_CHECK if a bounded loop of the unwrap
 * gave up or a frame did not join into one tree. */
odt_status odt_sino_read_status(const void *workspace, void *stream);

/* ---- Missing-apple-core correction ---------------------------------------
 * Replaces odtbrain.apple.correct (odtbrain/apple.py:113-263): iterative
 * filling of the apple core of the object function's spectrum with the
 * non-negativity ("nn") or symmetric-histogram ("sh") constraint, single-
 * precision 3D FFTs like the reference's pyFFTW plans.
 *   volume (n0, n1, n2) = the reconstruction's (Nx, Ny, Nx); n0 == n2
 *   f_real    device, n0*n1*n2 float32: the real part of f
 *   mask      device, n0*n1*n2 bytes (nonzero = use voxel) or NULL
 *   out       device, n0*n1*n2 complex64: the corrected object function
 *   gauss_weights  host, 2*gauss_radius+1 doubles: the 1D Gaussian of
 *             scipy.ndimage.gaussian_filter for sigma = max(shape)/100,
 *             truncate 4 (needed when enforce_envelope != 0)
 *   *iterations    iterations run before the stopping test ended the loop
 * Synchronous: it waits for `stream` between chunks of iterations. */
/* ODT_APPLE_NONE: no constraint (what the reference's loop does for any
 * other method name) */
enum odt_apple_method { ODT_APPLE_NN = 0, ODT_APPLE_SH = 1, ODT_APPLE_NONE = 2 };
typedef struct odt_apple_desc {
    int32_t n0, n1, n2;
    double res, nm;
    int32_t method;          /* odt_apple_method                           */
    double enforce_envelope; /* in [0, 1]; 0 disables the envelope         */
    int32_t max_iter;
    double min_diff;
    int32_t use_bg_shell;    /* background ellipsoid shell of width ...    */
    double bg_shell_width;   /* ... bg_shell_width                         */
    int32_t gauss_radius;
    const double *gauss_weights;
} odt_apple_desc;
odt_status odt_apple_workspace_size(const odt_apple_desc *desc, size_t *bytes);
/* Voxel flags of the correction (device, n0*n1*n2 bytes, stream-ordered):
 * bit 0 apple core (apple_core_3d, odtbrain/apple.py:8-53), bit 1 outside
 * the inscribed ellipsoid (spillover_region, :353-363), bit 2 background
 * shell (ellipsoid_shell, :281-286, when use_bg_shell), bit 3 mask.
 * workspace: odt_apple_flags_workspace_size bytes, 256-byte aligned. */
odt_status odt_apple_flags_workspace_size(const odt_apple_desc *desc,
                                          size_t *bytes);
odt_status odt_apple_flags(const odt_apple_desc *desc, const uint8_t *mask,
                           uint8_t *flags, void *workspace, void *stream);
odt_status odt_apple_correct(const odt_apple_desc *desc, const float *f_real,
                             const uint8_t *mask, void *out, void *workspace,
                             size_t workspace_bytes, int32_t *iterations,
                             void *stream);

/* One spatial constraint in place, replacing constraint_nn / constraint_sh
 * (odtbrain/apple.py:56-72, :75-110) called on their own.  Uses n0, n1, n2
 * (any 3D shape) and method (ODT_APPLE_NN or ODT_APPLE_SH) of the
 * descriptor.
 *   data      device, n0*n1*n2 values of real_bits (32 or 64) bits, or
 *             interleaved (re, im) pairs when is_complex: the real part is
 *             constrained, the imaginary part set to 0; arithmetic in the
 *             data's own precision like the reference's NumPy code
 *   mask      device bytes (nonzero = honour the voxel) or NULL
 *   bg_shell  device bytes (nonzero = known background) or NULL
 *   workspace odt_apple_constrain_workspace_size bytes, 256-byte aligned
 * Synchronous for ODT_APPLE_SH (the histogram's counts come to the host),
 * stream-ordered for ODT_APPLE_NN. */
odt_status odt_apple_constrain_workspace_size(const odt_apple_desc *desc,
                                              size_t *bytes);
odt_status odt_apple_constrain(const odt_apple_desc *desc, int32_t real_bits,
                               int32_t is_complex, void *data,
                               const uint8_t *mask, const uint8_t *bg_shell,
                               void *workspace, size_t workspace_bytes,
                               void *stream);

/* The Gaussian-blurred Fourier-amplitude envelope, replacing envelope_gauss
 * (odtbrain/apple.py:289-350) called on its own.  Uses n0, n1, n2 (n0 ==
 * n2), gauss_radius and gauss_weights of the descriptor.
 *   ftdata    device, n0*n1*n2 complex values (interleaved pairs of
 *             real_bits = 32 or 64 bits): the spectrum in FFT order
 *   core      device bytes, bit 0 set inside the apple core
 *   envelope  device, n0*n1*n2 values of real_bits bits (the type of the
 *             reference's |ftdata|)
 *   workspace odt_apple_envelope_workspace_size bytes, 256-byte aligned
 * Synchronous (a count decides whether the nearest-neighbour fill runs). */
odt_status odt_apple_envelope_workspace_size(const odt_apple_desc *desc,
                                             size_t *bytes);
odt_status odt_apple_envelope(const odt_apple_desc *desc, int32_t real_bits,
                              const void *ftdata, const uint8_t *core,
                              void *envelope, void *workspace,
                              size_t workspace_bytes, void *stream);

/* Wait for `stream`, then return ODT_ERR_DEVICE_CHECK if any kernel of this
 * plan recorded a failed internal check since the last call (the status word
 * is cleared). */
odt_status odt_bpp3d_read_status(const odt_bpp3d_plan *plan, void *stream);

odt_status odt_bpp3d_plan_destroy(odt_bpp3d_plan *plan);

/* ---- Failure injection (tests of the error paths) -------------------------
 * Neither call touches a kernel; no counterpart in the reference, whose
 * error paths are host-side checks only (odtbrain/_alg3d_bpp.py:237-258).
 *
 * odt_debug_inject_status: stream-ordered, sets the plan's device status
 * word to `bits` (0..255, the bits a kernel's own check records), exactly as
 * a kernel that tripped its check leaves it; the next odt_bpp3d_read_status
 * on that stream returns ODT_ERR_DEVICE_CHECK and clears it.
 *
 * odt_debug_set_table_alloc_limit: process-wide; odt_bpp3d_plan_create
 * returns ODT_ERR_OUT_OF_MEMORY, without calling cudaMalloc, when the plan's
 * device tables would exceed `bytes` (0 removes the limit). */
odt_status odt_debug_inject_status(const odt_bpp3d_plan *plan, int32_t bits,
                                   void *stream);
odt_status odt_debug_set_table_alloc_limit(uint64_t bytes);

/* Human-readable text of a status, and detail of the last host-side error
 * of the calling thread. */
const char *odt_status_string(odt_status status);
const char *odt_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* ODTBRAIN_GB300_H */
