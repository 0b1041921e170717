// Internal declarations shared by the stage kernels, the rotation kernels
// and the C-ABI layer.  Nothing here is part of the public interface.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace odt {

// Asynchronous global -> shared copies (cp.async: 16 bytes through L2 only,
// 8 bytes through L1) and their group bookkeeping.
#ifdef __CUDACC__
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
#endif

// Error bits recorded by kernels in the plan's device status word.
enum : int {
    DEVCHK_BOX_OVERFLOW = 1,   // a rotation footprint did not fit its tile
    DEVCHK_BAD_CONFIG = 2,     // a kernel was launched with an unsupported shape
    DEVCHK_COPY_TIMEOUT = 4    // a bulk tensor copy did not complete in time
};

// Number of boundary-correction terms of the B-spline prefilter that are
// applied; every pole (largest: order 5, |z| = 0.431) satisfies |z|^24 <
// 2e-9, below FP32 resolution of the corrected values.
constexpr int ZPOW_N = 24;

struct FilterTables {
    const float2 *G;      // [lNy*lNx] filter * prefilter particular factors
    const float2 *wsplit; // [lNy*lNx] propagator phase km*(M-1): (hi, lo)
    const float2 *step;   // [lNy*lNx] exp(i*km*(M-1))
    const float2 *alpha;  // [pole][lNy*lNx] z-prefilter boundary terms from p = 0
    const float2 *beta;   // [pole][lNy*lNx] z-prefilter boundary terms from p = nz-1
    const float2 *twx;    // [lNx] exp(-2 pi i m / lNx)
    const float2 *twy;    // [lNy] exp(-2 pi i m / lNy)
    const float *zpow;    // [pole][ZPOW_N] pole^m
};

struct StageParams {
    int A, ny, nx, nz, lNy, lNx, padyl, padxl;
    int pad_mode;
    float2 padval;
    int order;        // spline order; >= 2 means the prefilter is folded in
    int tilted;       // 1: 3D affine path (with a y-prefilter); 0: y-axis
                      //    path
    int in_c128;      // input sinogram is complex128
    int kx_zero_lo, kx_zero_hi;  // spectrum columns in [lo, hi) are all zero
                                 // (outside the |k| < km disc)
    float bx_ca, bx_cb;  // x-prefilter boundary solve (n = nx), one pole (adjoint)
    float by_ca, by_cb;  // y-prefilter boundary solve (n = ny; zero for ny = 1)
    int npoles;          // prefilter poles: 1 (orders 2, 3), 2 (orders 4, 5)
    float kxs[16];       // boundary solve of x lines: (A_i, B_i) = K d, 2np x 2np
    float kys[16];       // the same for y lines (tilted path)
    int ypitch;          // slab [a][z][x][y]: y pitch (yaxis_slab_pitch:
                         // ny rounded up to a multiple of 32, 1 for ny == 1)
    int col_slots;       // resident CTAs of the column stage on the device
    float zshift;        // plane p sits at z = p - nz/2 + zshift
    FilterTables tab;
    const float *gain;   // optional real per-frequency gain [lNy*lNx] (NULL: 1)
    const float2 *again; // optional complex per-angle gain [A][lNy*lNx], this
                         // batch's first angle at again (NULL: 1)
    int *status;
    // Tilted path, order >= 2 (ydefer = 1): the column stage leaves the
    // y-prefilter boundary terms to the row stage and stores the raw y-line samples around the crop's ends, 4
    // npoles rows of lNx per job (edge_row order), at T + yedge_off + (q -
    // q0) * 4 npoles * lNx of the job chunk's buffer T.
    int ydefer;
    long long yedge_off;
};

// y pitch of the slab layout [a][z][x][y]
// y pitch of the y-axis coefficient slab [a][z][x][y]: a multiple of 32,
// except for single-row planes (the 2D reconstruction), stored as [a][z][x]
inline int yaxis_slab_pitch(int ny) { return ny == 1 ? 1 : (ny + 31) / 32 * 32; }

struct RotParams {
    int ny, nx, nz;
    int ypitch;       // slab y pitch (yaxis_slab_pitch)
    int nbatch_angles;
    int first_pass;   // this launch starts the sum (overwrite)
    int last_pass;    // this launch ends the sum (drop the compensation)
    int onlyreal;
    int *status;
};

// Launchers (stream-ordered; return cudaGetLastError()).
cudaError_t launch_rows_forward(const StageParams &P, const void *sino_batch, const double *weights_batch,
                                int nb, float2 *rowspec, cudaStream_t s);
cudaError_t launch_columns_propagate(const StageParams &P, const float2 *rowspec, float2 *T, int q0, int qn,
                                     cudaStream_t s);
// z-prefilter boundary columns of a batch (order >= 2): Tab[a][2][ny][lNx].
cudaError_t launch_columns_boundary(const StageParams &P, const float2 *rowspec, float2 *Tab, int nb,
                                    cudaStream_t s);
// Single-row planes (lNy == ny == 1, slab pitch 1): the column and row
// stages fused in one launch over jobs [q0, q0 + qn), from the row spectra.
bool single_row_plan(const StageParams &P);
// Square power-of-two padded planes (N >= 256) cropped to their centred
// half (ny = nx = N/2 from N/4): the column and row stages then run
// kernels whose crop and edge positions are compile-time constants.
bool half_crop(const StageParams &P);
cudaError_t launch_rows_line(const StageParams &P, const float2 *rowspec, const float2 *Tab, float2 *slab, int q0,
                             int qn, cudaStream_t s);
cudaError_t launch_rows_inverse(const StageParams &P, const float2 *T, const float2 *Tab, float2 *slab, int q0,
                                int qn, cudaStream_t s);
// Scratch (device bytes) the rotation stage needs for a batch: per-(angle,
// tile) geometry records of the y-axis path.
size_t rotate_scratch_bytes(int nbatch_angles, int ny, int nx, int nz, int tilted);
cudaError_t launch_rotate(const RotParams &R, int order, int tilted, const float2 *slab, const double *geo,
                          void *volume, float2 *comp, void *scratch, cudaStream_t s);
cudaError_t configure_kernels(const StageParams &P);
// Resident CTAs (all SMs) of the column-stage kernel for these sizes.
int columns_slots(const StageParams &P);
cudaError_t configure_rotate_kernels();

// Adjoint (adjoint.cu, rotate.cu).
cudaError_t configure_adjoint_kernels(const StageParams &P);
// Scratch: rotate_scratch_bytes(batch, ...) (one 64-byte record per angle and
// 16 x 16 tile, like the forward).  vol_grad: the volume gradient in the
// [z][x][y] order (launch_volume_zxy) for the y axis, [z][y][x] for the
// tilted geometry.
cudaError_t launch_rotate_adjoint(const RotParams &R, int order, int tilted, const float2 *vol_grad,
                                  const double *geo, float2 *slab_grad, void *scratch, cudaStream_t s);
// The volume gradient [z][y][x] in the [z][x][y] order that the y-axis
// resampling transpose reads (y innermost, one contiguous run per output).
cudaError_t launch_volume_zxy(const float2 *vol, float2 *vol_zxy, int nz, int ny, int nx, cudaStream_t s);
cudaError_t configure_rotate_adjoint_kernels();
cudaError_t launch_adj_rows(const StageParams &P, const float2 *sgrad, float2 *Tg, int q0, int qn, cudaStream_t s);
cudaError_t launch_adj_columns(const StageParams &P, const float2 *Tg, float2 *Qg, int q0, int qn, cudaStream_t s);
cudaError_t launch_adj_spectrum(const StageParams &P, const float2 *rowspec, const float2 *Qg, float *dgain,
                                float2 *dagain, float2 *W, int nb, cudaStream_t s);
cudaError_t launch_adj_rows_full(const StageParams &P, const float2 *W, float2 *Pg, int nb, cudaStream_t s);
cudaError_t launch_adj_pad(const StageParams &P, const float2 *Pg, const double *weights, int nb, float2 *dsino,
                           cudaStream_t s);
bool line_size_supported(int n);

// Record `msg` as the calling thread's last error (odt_last_error) and
// return `status`.
int set_error(int status, const char *msg);

}  // namespace odt
