// Filter stages (a) and (b) of the 3D backpropagation on sm_103a.
//
// Reference loop body (odtbrain/_alg3d_bpp.py:492-528, _alg3d_bppt.py:
// 865-898), per angle:
//   pad -> forward 2D FFT -> *prefactor/(lNx*lNy) -> for every z plane p:
//   *exp(i km (M-1) z_p) -> unnormalised backward 2D FFT -> crop.
//
// GB300 decomposition (three kernels, all lines in registers):
//   rows_forward       padded+weighted rows, forward FFT along x
//   columns_propagate  forward FFT along y, filter multiply, then for a run
//                      of z planes: propagator (exact anchor + complex
//                      recurrence), backward FFT along y, crop in y
//   rows_inverse       backward FFT along x, crop in x -> coefficient slab
//
// The B-spline prefilter that scipy.ndimage applies before resampling
// (mirror boundaries, along z and x of every plane; along all three axes on
// the tilted path) is folded into these stages exactly: each Fourier
// component exp(i k n) of a cropped line has the prefiltered form
// exp(i k n)/Bhat(k) + A z^n + B z^(N-1-n) (z the spline pole, Bhat the
// sampled B-spline's transfer function), where A and B follow from the two
// mirror conditions.  So the spectrum is divided by Bhat along every
// prefiltered axis (folded into the filter table G), z gets per-frequency
// boundary terms (alpha, beta tables), and x (and y) get per-line boundary
// terms computed from four samples just outside the crop.
#include <algorithm>
#include <type_traits>

#include "odt_fft.cuh"
#include "odt_internal.cuh"
#include "odt_stage_util.cuh"

namespace odt {

// Column stage of half-crop plans: keep the propagator step exp(i w) of a
// thread's elements in registers instead of shared memory, and read the
// third radix-8 pass's twiddles from the per-thread-class table (256^3
// workload: 25.7 ms without either, 25.7 / 26.0 ms with one of them,
// 24.1 ms with both).
constexpr bool kColumnStepRegs = true;
constexpr bool kColumnTw2 = true;
// Planes between exact propagator anchors within a column CTA's run.
constexpr int kReanchorPlanes = 32;
// The half-crop column kernel's shared memory (smem_cols_half) has one
// [n][KX] region, which holds the filtered spectrum because the steps are
// in registers.
static_assert(kColumnStepRegs, "smem_cols_half assumes register-held propagator steps");
// Column CTAs that run through up to 256 planes of an angle, re-anchoring
// the propagator every kReanchorPlanes planes: power-of-two columns of
// 64-thread lines with the steps in registers (4 columns per CTA, the
// 512-point planes).  256^3 workload,
// cap on the planes per CTA against the column stage: 32 planes 24.1 ms,
// 64 22.8, 128 22.4, 256 22.2 ms.  The other column kernels keep runs of
// at most kReanchorPlanes planes (one exact anchor each): the 512-thread
// CTAs of 256-point columns lost 30 % with longer runs (one wave of long
// CTAs), and the generic kernel's extra shared memory for the re-anchoring
// cost more than the longer runs saved.
template <class L, int KX, bool HALF>
constexpr bool long_runs()
{
    return pow2_len<L>() > 0 && kColumnStepRegs && KX * L::TPL <= 256;
}
// Column kernels that hold the propagator steps in registers and read the
// third pass's twiddles from the 64x7 table (N >= 512): the half-crop
// kernel, and for other crops power-of-two columns in CTAs of at most 256
// threads (with more threads per CTA, 64 registers per thread, the steps
// spill).
template <class L, int KX, bool HALF>
constexpr bool column_regs()
{
    return kColumnStepRegs && (HALF || (pow2_len<L>() > 0 && KX * L::TPL <= 256));
}

// ---------------------------------------------------------------------------
// (a) rows: pad + weight + forward FFT along x.
// rowspec[a][y][kx], a in the batch, y over the padded height.
template <class L, int LPC>
__global__ void __launch_bounds__(LPC * L::TPL) k_rows_forward(StageParams P, L line, const void *sino,
                                                               const double *weights, int nb, float2 *rowspec)
{
    extern __shared__ float2 smem[];
    const int n = line.size();
    const int ls = xslots<false>(n);
    float2 *buf0 = smem, *buf1 = smem + LPC * ls, *tw = smem + 2 * LPC * ls;
    copy_twiddles<L>(tw, P.tab.twx, n);
    const int l = threadIdx.x / L::TPL, j = threadIdx.x % L::TPL;
    const int lid = (int)blockIdx.x * LPC + l;
    const int nlines = nb * P.lNy;
    const bool valid = lid < nlines;
    const int a = valid ? lid / P.lNy : 0;
    const int y = valid ? lid - a * P.lNy : 0;
    const double w = weights ? weights[a] : 1.0;
    const size_t arow = (size_t)a * P.ny * P.nx;
    float2 v[L::SLOTS];
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int x = j + r * L::TPL;
        v[r] = (valid && x < n) ? padded_sample(P, sino, arow, w, y, x) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    int flip = 0;
    line.template run<-1>(v, j, buf0 + l * ls, buf1 + l * ls, 1, tw, flip);
    if (!valid)
        return;
    float2 *dst = rowspec + (size_t)lid * n;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int x = j + r * L::TPL;
        if (x < n)
            dst[x] = v[r];
    }
}

// ---------------------------------------------------------------------------
// Column helpers shared by the two column kernels.  A CTA owns KX adjacent
// spectrum columns kx; thread (c, j) holds rows ky = j + r*TPL of column c.

// Column kx of angle a's row spectra, forward FFT along y, times the filter
// table G (which includes the prefilter particular factors).
template <class L, int KX>
__device__ __forceinline__ void column_spectrum(const StageParams &P, const L &line, const float2 *rowspec, int a,
                                                int kx, bool colok, int c, int j, float2 *buf0, float2 *buf1,
                                                const float2 *tw, int &flip, float2 (&v)[L::SLOTS])
{
    const int n = line.size();
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int ky = j + r * L::TPL;
        v[r] = (colok && ky < n) ? rowspec[((size_t)a * n + ky) * P.lNx + kx] : make_float2(0.f, 0.f);
    }
    line.template run<-1, true>(v, j, buf0 + c, buf1 + c, KX, tw, flip);
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int ky = j + r * L::TPL;
        if (colok && ky < n) {
            const size_t k = (size_t)ky * P.lNx + kx;
            v[r] = cmul(v[r], P.tab.G[k]);
            if (P.gain)
                v[r] = cscale(v[r], P.gain[k]);
            if (P.again)
                v[r] = cmul(v[r], P.again[(size_t)a * P.lNy * P.lNx + k]);
        } else {
            v[r] = make_float2(0.f, 0.f);
        }
    }
}

// The edge samples of the y-prefilter solve that thread j holds after a
// column's backward transform: bit 8 r + e is set when slot r holds the
// sample of edge slot e (the same for every plane of the CTA, so it is
// computed once).  Power-of-two lines (8 slots).
template <class L, int NP>
__device__ __forceinline__ unsigned long long edge_holdings(const StageParams &P, int n, int j)
{
    unsigned long long m = 0;
#pragma unroll
    for (int e = 0; e < EDGE_SLOTS; ++e) {
        if (edge_used(e, NP)) {
            const int pos = (P.padyl + edge_offset(e, P.ny) + 2 * n) % n;
            if (pos % L::TPL == j)
                m |= 1ull << (8 * (pos / L::TPL) + e);
        }
    }
    return m;
}

// Backward FFT along y of v, then the y-prefilter boundary terms (YF > 0:
// tilted path, order >= 2, YF poles) and the cropped store dst[yy * lNx]
// for yy < ny.  DEFER (P.ydefer): the terms' coefficients need the line's
// edge samples, held by a few other threads, so adding them here costs a
// barrier per line; instead the raw edge samples go to yedge[row * lNx]
// (rows edge_row(e)), the crop is stored raw, and the row stage adds the
// terms.  `eheld`: edge_holdings of this thread (power-of-two lines).
template <class L, int KX, int YF, bool TW2 = false, bool DEFER = false>
__device__ __forceinline__ void column_inverse_store(const StageParams &P, const L &line, float2 (&v)[L::SLOTS],
                                                     int c, int j, bool colok, float2 *buf0, float2 *buf1,
                                                     const float2 *tw, float2 *edge, int &flip, float2 *dst,
                                                     float2 *yedge = nullptr, unsigned long long eheld = 0)
{
    const int n = line.size();
    const int ny = P.ny, padyl = P.padyl;
    line.template run<1, true, TW2>(v, j, buf0 + c, buf1 + c, KX, tw, flip);
    constexpr bool yfix = YF > 0 && !DEFER;
    constexpr int NPY = YF > 0 ? YF : 1;
    float2 cf[2 * NPY];
    if constexpr (YF > 0 && DEFER) {
        if constexpr (L::SLOTS <= 8) {
            if (eheld && colok) {
#pragma unroll
                for (int r = 0; r < L::SLOTS; ++r) {
                    const unsigned m = (unsigned)(eheld >> (8 * r)) & 0xffu;
                    if (m) {
#pragma unroll
                        for (int e = 0; e < EDGE_SLOTS; ++e)
                            if (edge_used(e, NPY) && (m & (1u << e)))
                                yedge[(size_t)edge_row(e, NPY) * P.lNx] = v[r];
                    }
                }
            }
        } else if (colok) {
#pragma unroll
            for (int e = 0; e < EDGE_SLOTS; ++e) {
                float2 t;
                if (edge_used(e, NPY) && held<L>(v, j, (padyl + edge_offset(e, ny) + 2 * n) % n, t))
                    yedge[(size_t)edge_row(e, NPY) * P.lNx] = t;
            }
        }
    }
    if constexpr (yfix) {
        // u around the crop's ends (periodic over the padded height)
#pragma unroll
        for (int e = 0; e < EDGE_SLOTS; ++e) {
            float2 t;
            if (edge_used(e, NPY) && held<L>(v, j, (padyl + edge_offset(e, ny) + 2 * n) % n, t))
                edge[c * EDGE_SLOTS + e] = t;
        }
        __syncthreads();
        pf_coefs<NPY>(P.kys, edge + c * EDGE_SLOTS, cf);
    }
    if (!colok)
        return;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int yy = j + r * L::TPL - padyl;
        if (yy >= 0 && yy < ny) {
            float2 o = v[r];
            if constexpr (yfix)
                o = pf_apply<NPY>(P, cf, yy, ny, o);
            dst[(size_t)yy * P.lNx] = o;
        }
    }
}

// Half-crop form of column_inverse_store (half_crop plans: ny = N/2 rows
// starting at N/4 of a power-of-two column of N).  Thread j then holds the
// cropped rows in slots 2..5, row j + TPL*(r-2), and the four edge samples
// of the y-prefilter solve at compile-time slots, so the crop needs no
// predicates and the stores use constant offsets from one row pointer.
// dst points at row 0 of the job's T block, column kx (row stride N).
// DEFER (P.ydefer): as in column_inverse_store, the raw edge samples go to
// yedge[row * N] (their holders and slots are compile-time here) and the
// row stage adds the y-prefilter terms.
template <class L, int KX, int YF, bool TW2, bool DEFER = false>
__device__ __forceinline__ void column_inverse_store_half(const StageParams &P, const L &line, float2 (&v)[L::SLOTS],
                                                          int c, int j, float2 *buf0, float2 *buf1,
                                                          const float2 *tw, float2 *edge, int &flip, float2 *dst,
                                                          float2 *yedge = nullptr)
{
    constexpr int N = L::N, TPL = L::TPL, NY = N / 2, PAD = N / 4;
    line.template run<1, true, TW2>(v, j, buf0 + c, buf1 + c, KX, tw, flip);
    if constexpr (YF > 0 && DEFER) {
#pragma unroll
        for (int e = 0; e < EDGE_SLOTS; ++e) {
            if (edge_used(e, YF)) {
                const int pos = PAD + edge_offset(e, NY);
                if (j == pos % TPL)
                    yedge[(size_t)edge_row(e, YF) * N] = v[pos / TPL];
            }
        }
    } else if constexpr (YF > 0) {
        // y-prefilter boundary terms from u around the crop's ends
        // (compile-time positions)
#pragma unroll
        for (int e = 0; e < EDGE_SLOTS; ++e) {
            float2 t;
            if (edge_used(e, YF) && held<L>(v, j, PAD + edge_offset(e, NY), t))
                edge[c * EDGE_SLOTS + e] = t;
        }
        __syncthreads();
        float2 cf[2 * YF];
        pf_coefs<YF>(P.kys, edge + c * EDGE_SLOTS, cf);
#pragma unroll
        for (int r = 2; r <= 5; ++r)
            v[r] = pf_apply<YF>(P, cf, j + TPL * (r - 2), NY, v[r]);
    }
    float2 *d = dst + (size_t)j * N;
#pragma unroll
    for (int r = 2; r <= 5; ++r)
        d[(r - 2) * TPL * N] = v[r];
}

// ---------------------------------------------------------------------------
// (b0) z-prefilter boundary columns, once per angle (order >= 2).  The
// prefiltered propagator of plane p is E_p + alpha z^p + beta z^(nz-1-p);
// by linearity the alpha and beta parts are transformed once here
// (Tab[a][0] = column transform of G*alpha, Tab[a][1] of G*beta) and the row
// stage adds z^p Tab[a][0] + z^(nz-1-p) Tab[a][1] to the first and last
// planes' rows.
template <class L, int KX, int YF>
__global__ void __launch_bounds__(KX * L::TPL) k_columns_boundary(StageParams P, L line, const float2 *rowspec,
                                                                  float2 *Tab)
{
    if (!group_active<KX>(P, blockIdx.x * KX))
        return;  // all-zero columns: the row stage never reads them
    extern __shared__ float2 smem[];
    const int n = line.size();
    const int ls = xslots<true>(n);
    float2 *buf0 = smem, *buf1 = smem + KX * ls, *tw = smem + 2 * KX * ls, *edge = tw + tw_slots(n);
    copy_twiddles<L>(tw, P.tab.twy, n);
    const int c = threadIdx.x % KX, j = threadIdx.x / KX;
    const int kx = blockIdx.x * KX + c;
    const bool colok = kx < P.lNx;
    const int a = blockIdx.y;
    __syncthreads();
    int flip = 0;
    float2 g[L::SLOTS];
    column_spectrum<L, KX>(P, line, rowspec, a, kx, colok, c, j, buf0, buf1, tw, flip, g);
    const int np = P.npoles;
    const size_t K = (size_t)P.lNy * P.lNx;
#pragma unroll 1
    for (int t = 0; t < 2 * np; ++t) {
        const float2 *tab = t < np ? P.tab.alpha + t * K : P.tab.beta + (t - np) * K;
        float2 v[L::SLOTS];
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int ky = j + r * L::TPL;
            v[r] = (colok && ky < n) ? cmul(g[r], tab[(size_t)ky * P.lNx + kx]) : make_float2(0.f, 0.f);
        }
        column_inverse_store<L, KX, YF>(P, line, v, c, j, colok, buf0, buf1, tw, edge, flip,
                                        Tab + ((size_t)(a * 2 * np + t) * P.ny) * P.lNx + kx);
    }
}

// (b1) columns: for the z planes of jobs q in [q0, q0+qn) (q = a*nz + p):
// propagator (exact anchor, then a complex recurrence whose per-element step
// lives in shared memory), backward FFT along y, crop.  Output
// T[q-q0][y][kx], y over the cropped height.
template <class L, int KX, bool HALF, int YF>
__global__ void __launch_bounds__(KX * L::TPL, (KX * L::TPL <= 256) ? 3 : ((KX * L::TPL <= 512) ? 2 : 1))
    k_columns_propagate(StageParams P, L line, const float2 *rowspec, float2 *T, int q0, int qn, int ppc)
{
    if (!group_active<KX>(P, blockIdx.x * KX))
        return;  // all-zero columns: the row stage never reads them
    // power-of-two columns: the per-element propagator step lives in
    // registers and (N >= 512) the third radix-8 pass reads
    // per-thread-class twiddles (with long runs, tilted 200^3 step 72.1 ->
    // 70.6 ms; same box)
    constexpr bool STEP_REGS = column_regs<L, KX, HALF>();
    constexpr bool TW2 = STEP_REGS && kColumnTw2 && pow2_len<L>() >= 512;
    extern __shared__ float2 smem[];
    const int n = line.size();  // lNy
    const int ls = xslots<true>(n);
    float2 *buf0 = smem, *buf1 = smem + KX * ls, *tw = smem + 2 * KX * ls;
    float2 *edge = tw + (TW2 ? tw_slots2(n) : tw_slots(n)); // [KX][EDGE_SLOTS]
    float2 *stp = edge + EDGE_SLOTS * KX;  // [n][KX] propagator step per element
    // long runs: [n][KX] the filtered spectrum G X of the current angle,
    // for the exact re-anchoring every kReanchorPlanes planes (in the step
    // region: the steps live in registers)
    constexpr bool REANCHOR = long_runs<L, KX, HALF>();
    float2 *gx = stp;
    if constexpr (TW2)
        copy_twiddles2<L>(tw, P.tab.twy, n);
    else
        copy_twiddles<L>(tw, P.tab.twy, n);
    const int c = threadIdx.x % KX, j = threadIdx.x / KX;
    const int kx = blockIdx.x * KX + c;
    const bool colok = kx < P.lNx;
    const int lNx = P.lNx, nz = P.nz, ny = P.ny;
    const int qb = q0 + blockIdx.y * ppc;
    const int qe = min(q0 + qn, qb + ppc);
    float2 St[L::SLOTS];  // STEP_REGS: exp(i w) of this thread's elements
    if constexpr (STEP_REGS) {
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r)  // (columns beyond lNx: never stored)
            St[r] = colok ? P.tab.step[(size_t)(j + r * L::TPL) * lNx + kx] : make_float2(1.f, 0.f);
    }
    __syncthreads();

    float2 V[L::SLOTS];  // G * exp(i w z_p) for this thread's elements
    int flip = 0;
    // tilted generic crops: the edge samples this thread holds (fixed)
    unsigned long long eheld = 0;
    if constexpr (!HALF && YF > 0 && L::SLOTS <= 8)
        eheld = edge_holdings<L, YF>(P, n, j);
    int cur_a = -1;
    int since = 0;  // planes advanced by the recurrence since the last exact anchor
    int a = qb / nz, p = qb % nz;
    for (int q = qb; q < qe; ++q, ++p) {
        if (p == nz) {
            p = 0;
            ++a;
        }
        if (a != cur_a || (REANCHOR && since == kReanchorPlanes)) {
            // exact anchor at the first plane of an angle, and again every
            // kReanchorPlanes planes: the FP32 recurrence drifts by about one
            // rounding per plane (measured on the 256^3 workload: rel-L2 to
            // the FP64 oracle 3.5e-7 with anchors every 32 planes, 1.6e-6
            // with one anchor per 256-plane run)
            const bool fresh = a != cur_a;
            if (fresh)
                column_spectrum<L, KX>(P, line, rowspec, a, kx, colok, c, j, buf0, buf1, tw, flip, V);
            const float zp = (float)p - 0.5f * (float)nz + P.zshift;
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int ky = j + r * L::TPL;
                if (colok && ky < n) {
                    const size_t k = (size_t)ky * lNx + kx;
                    if (fresh) {
                        if (REANCHOR)
                            gx[ky * KX + c] = V[r];  // read back only by this thread
                        if (!STEP_REGS)
                            stp[ky * KX + c] = P.tab.step[k];
                    } else if (REANCHOR) {
                        V[r] = gx[ky * KX + c];
                    }
                    V[r] = cmul(V[r], expi_phase(P.tab.wsplit[k], zp));
                }
            }
            cur_a = a;
            since = 0;
        }
        ++since;
        float2 v[L::SLOTS];
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            v[r] = V[r];
            const int ky = j + r * L::TPL;
            if constexpr (STEP_REGS)
                V[r] = cmul(V[r], St[r]);  // (ky < n: a power-of-two line)
            else if (HALF || ky < n)  // half-crop plans: a power-of-two line, ky < n
                V[r] = cmul(V[r], stp[ky * KX + c]);
        }
        if constexpr (HALF)  // (tilted: the y-prefilter terms go to the row stage)
            column_inverse_store_half<L, KX, YF, TW2, (YF > 0)>(
                P, line, v, c, j, buf0, buf1, tw, edge, flip, T + (size_t)(q - q0) * (L::N / 2) * L::N + kx,
                T + P.yedge_off + (size_t)(q - q0) * 4 * (YF > 0 ? YF : 1) * L::N + kx);
        else if constexpr (YF > 0)  // (tilted: the y-prefilter terms go to the row stage)
            column_inverse_store<L, KX, YF, TW2, true>(
                P, line, v, c, j, colok, buf0, buf1, tw, edge, flip, T + (size_t)(q - q0) * ny * lNx + kx,
                T + P.yedge_off + (size_t)(q - q0) * 4 * YF * lNx + kx, eheld);
        else
            column_inverse_store<L, KX, YF, TW2>(P, line, v, c, j, colok, buf0, buf1, tw, edge, flip,
                                             T + (size_t)(q - q0) * ny * lNx + kx);
    }
}

// ---------------------------------------------------------------------------
// (b2) rows: (+ z-boundary rows), backward FFT along x, x-prefilter boundary
// terms, crop -> slab.
// Slab layout [a][z][x][y] (both geometries) with the y pitch P.ypitch (a
// multiple of 32, or 1 for single-row planes).  A CTA owns RG consecutive y rows of one plane (job) and
// transforms them in groups of LPC lines (one line per TPL threads); the T
// values of the next group are loaded (evict-first) into registers while
// the current group is transformed.  When a line is whole warps its FFT
// exchanges sync only its own warps (named barrier).  The cropped rows of a
// group are transposed through shared memory and stored as runs of LPC
// consecutive y per x (rows y >= ny of a group are zero; groups and CTAs
// wholly beyond ny are not run).
template <int LPC>
constexpr int rows_per_cta()
{
    return LPC >= 8 ? LPC : 8;
}

// YD (P.ydefer): the column stage left the tilted path's y-prefilter
// boundary terms to this stage.  A CTA with rows within ZPOW_N of either end
// of the crop solves each column's coefficients once, from the job's raw
// edge samples, into shared memory (lines of up to 2048; longer lines solve
// them per row), and those rows add the terms before the z-boundary rows:
// the same values in the same order as in the column stage.
template <class L>
constexpr bool ycoef_smem()
{
    return pow2_len<L>() == 0 || pow2_len<L>() <= 2048;
}
template <class L, int NP, bool YD>
constexpr size_t smem_rows_y(int n)
{
    return (YD && ycoef_smem<L>()) ? (size_t)2 * NP * n * sizeof(float2) : 0;
}
template <class L, int LPC, int NP, bool YD>
__global__ void __launch_bounds__(LPC * L::TPL, (LPC * L::TPL <= 256) ? 4 : 1)
    k_rows_inverse(StageParams P, L line, const float2 *T, const float2 *Tab, float2 *slab, int q0, int qn)
{
    constexpr int RG = rows_per_cta<LPC>(), G = RG / LPC;
    extern __shared__ float2 smem[];
    const int n = line.size();  // lNx
    const int ls = xslots<false>(n);
    float2 *buf0 = smem, *buf1 = smem + LPC * ls, *tw = smem + 2 * LPC * ls;
    copy_twiddles<L>(tw, P.tab.twx, n);
    const int l = threadIdx.x / L::TPL, j = threadIdx.x % L::TPL;
    // lines of whole warps sync on named barrier 1 + l
    const int bar = (L::TPL % 32 == 0 && LPC < 15) ? 1 + l : 0;
    const int ny = P.ny, nx = P.nx, nz = P.nz, padxl = P.padxl, yp = P.ypitch;
    const int cpj = (ny + RG - 1) / RG;  // CTAs per job (rows y < ny only)
    const int qrel = (int)blockIdx.x / cpj;
    const int ybase = ((int)blockIdx.x - qrel * cpj) * RG;
    // groups holding at least one row y < ny (the slab rows y >= ny are
    // never read: the resampling lanes of those y store nothing)
    const int GV = min(G, (ny - ybase + LPC - 1) / LPC);
    const int qq = q0 + qrel;  // the grid covers exactly qn jobs
    const int a = qq / nz, p = qq - a * nz;
    const bool pf = P.order >= 2;
    constexpr int np = NP;
    // z-boundary weights of this plane: z_i^p (alpha rows), z_i^(nz-1-p)
    // (beta rows), per pole
    float zl[2], zh[2];
    bool zb_any = false;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        zl[i] = (pf && i < np && p < ZPOW_N) ? P.tab.zpow[i * ZPOW_N + p] : 0.f;
        zh[i] = (pf && i < np && nz - 1 - p < ZPOW_N) ? P.tab.zpow[i * ZPOW_N + nz - 1 - p] : 0.f;
        zb_any = zb_any || zl[i] != 0.f || zh[i] != 0.f;
    }
    const float2 *Tq = T + (size_t)qrel * ny * n;
    float2 *dst = slab + ((size_t)a * nz + p) * nx * yp + ybase;
    // this thread's T values of row y (zeros for y >= ny or zero columns)
    auto load_row = [&](int y, float2 (&v)[L::SLOTS]) {
        const bool valid = y < ny;
        const float2 *src = Tq + (size_t)(valid ? y : 0) * n;
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int x = j + r * L::TPL;
            v[r] = (valid && column_active(P, x)) ? __ldcs(src + x) : make_float2(0.f, 0.f);
        }
    };
    // YD: the y-prefilter coefficient rows of this job, [2 NP][n] after the
    // row buffers (CTAs with boundary rows)
    float2 *ycs = smem + (2 * LPC * ls + tw_slots(n) + EDGE_SLOTS * LPC);
    const float2 *yed = T + P.yedge_off + (size_t)qrel * 4 * NP * n;
    if constexpr (YD && ycoef_smem<L>()) {
        if (ybase < ZPOW_N || min(ybase + RG, ny) - 1 >= ny - ZPOW_N) {
            for (int x = threadIdx.x; x < n; x += LPC * L::TPL) {
                float2 cy[2 * NP];
                if (column_active(P, x)) {
                    float2 ed[EDGE_SLOTS];
#pragma unroll
                    for (int e = 0; e < EDGE_SLOTS; ++e)
                        ed[e] = edge_used(e, NP) ? yed[(size_t)edge_row(e, NP) * n + x] : make_float2(0.f, 0.f);
                    pf_coefs<NP>(P.kys, ed, cy);
                } else {
#pragma unroll
                    for (int i = 0; i < 2 * NP; ++i)
                        cy[i] = make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int i = 0; i < 2 * NP; ++i)
                    ycs[i * n + x] = cy[i];
            }
        }
    }
    float2 v[L::SLOTS], vn[L::SLOTS];
    load_row(ybase + l, v);
    __syncthreads();  // twiddles (and the coefficient rows)
#pragma unroll 1
    for (int g = 0; g < GV; ++g) {
        const int y = ybase + g * LPC + l;
        const bool valid = y < ny;
        if (g + 1 < GV)
            load_row(y + LPC, vn);
        if constexpr (YD) {
            if (valid && (y < ZPOW_N || ny - 1 - y < ZPOW_N)) {
#pragma unroll
                for (int r = 0; r < L::SLOTS; ++r) {
                    const int x = j + r * L::TPL;
                    if (column_active(P, x)) {
                        float2 cy[2 * NP];
                        if constexpr (ycoef_smem<L>()) {
#pragma unroll
                            for (int i = 0; i < 2 * NP; ++i)
                                cy[i] = ycs[i * n + x];
                        } else {
                            float2 ed[EDGE_SLOTS];
#pragma unroll
                            for (int e = 0; e < EDGE_SLOTS; ++e)
                                ed[e] = edge_used(e, NP) ? yed[(size_t)edge_row(e, NP) * n + x]
                                                         : make_float2(0.f, 0.f);
                            pf_coefs<NP>(P.kys, ed, cy);
                        }
                        v[r] = pf_apply<NP>(P, cy, y, ny, v[r]);
                    }
                }
            }
        }
        if (valid && zb_any) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                if (i < np) {
                    const float2 *ta = Tab + ((size_t)(a * 2 * np + i) * ny + y) * n;
                    const float2 *tb = Tab + ((size_t)(a * 2 * np + np + i) * ny + y) * n;
#pragma unroll
                    for (int r = 0; r < L::SLOTS; ++r) {
                        const int x = j + r * L::TPL;
                        if (column_active(P, x)) {
                            const float2 u = ta[x], w = tb[x];
                            v[r] = make_float2(fmaf(zh[i], w.x, fmaf(zl[i], u.x, v[r].x)),
                                               fmaf(zh[i], w.y, fmaf(zl[i], u.y, v[r].y)));
                        }
                    }
                }
            }
        }
        int flip = 0;
        line.template run<1>(v, j, buf0 + l * ls, buf1 + l * ls, 1, tw, flip, bar);
        float2 cf[2 * NP];
        if (pf) {
            // the line's samples around the crop's ends (periodic): every
            // thread writes its values to the exchange buffer the FFT's last
            // exchange did not use (its reads ended before that exchange's
            // barrier), then each thread reads the edge samples
            // (plain positions 0..n-1: within the line's slots for every
            // line type, and conflict-free for these stride-1 writes)
            float2 *sc = (flip ? buf1 : buf0) + l * ls;
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int x = j + r * L::TPL;
                if (x < n)
                    sc[x] = v[r];
            }
            if (bar > 0)
                line_sync(bar, L::TPL);
            else
                __syncthreads();
            float2 ed[EDGE_SLOTS];
#pragma unroll
            for (int e = 0; e < EDGE_SLOTS; ++e)
                ed[e] = edge_used(e, np) ? sc[(padxl + edge_offset(e, nx) + 2 * n) % n] : make_float2(0.f, 0.f);
            pf_coefs<NP>(P.kxs, ed, cf);
        }
        // stage[x][l] (pitch LPC+1) in buf0, then runs of LPC y per x
        __syncthreads();  // every line is done with buf0
        float2 *stage = buf0;
        constexpr int SP = LPC + 1;
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int xx = j + r * L::TPL - padxl;
            if (xx >= 0 && xx < nx) {
                float2 o = v[r];
                if (pf)
                    o = pf_apply<NP>(P, cf, xx, nx, o);
                stage[xx * SP + l] = valid ? o : make_float2(0.f, 0.f);
            }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < nx * LPC; e += LPC * L::TPL) {
            const int xx = e / LPC, ll = e - xx * LPC;
            if (ybase + g * LPC + ll < ny)  // pitch 1 for single-row planes
                __stcs(dst + (size_t)xx * yp + g * LPC + ll, stage[xx * SP + ll]);
        }
        if (g + 1 < GV) {
            __syncthreads();  // stage reads done before buf0 is reused
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r)
                v[r] = vn[r];
        }
    }
}

// (b2, half-crop plans) k_rows_inverse for square power-of-two planes
// whose crop is the centred half (nx = ny = N/2 from N/4; the slab y pitch
// is then N/2): every position the row needs -- the cropped outputs (slots
// 2..5 of thread j, x = j + TPL*(r-2)), the x-prefilter edge samples and
// the rows with boundary terms -- is a compile-time function of the thread
// and slot, so the row runs without per-element index arithmetic or crop
// predicates.  The all-zero spectrum columns (outside the |k| < km disc,
// not written by the column stage) are a per-thread slot mask computed
// once.  A CTA owns LPC*G consecutive rows of one job, LPC lines at a time.
// YD (P.ydefer): the tilted path's y-prefilter terms, added as in
// k_rows_inverse.
template <class L, int LPC, int G, int NP, bool YD>
__global__ void __launch_bounds__(LPC * L::TPL, (LPC * L::TPL <= 256) ? 4 : 1)
    k_rows_inverse_half(StageParams P, L line, const float2 *T, const float2 *Tab, float2 *slab, int q0)
{
    constexpr int N = L::N, TPL = L::TPL, NX = N / 2, PAD = N / 4, RG = LPC * G, CPJ = NX / RG;
    static_assert(NX % RG == 0, "rows per CTA must divide the crop");
    extern __shared__ float2 smem[];
    constexpr int ls = xslots<false>(N);
    float2 *buf0 = smem, *buf1 = smem + LPC * ls, *tw = smem + 2 * LPC * ls;
    float2 *edge = tw + tw_slots(N);  // [LPC][EDGE_SLOTS]
    // (the third-pass twiddle table costs more to set up per CTA than its
    // conflict-free reads save here: +0.7 ms for the 256^3 row stage)
    copy_twiddles<L>(tw, P.tab.twx, N);
    const int l = threadIdx.x / TPL, j = threadIdx.x % TPL;
    const int bar = 1 + l;  // each line is whole warps (TPL >= 32)
    const int nz = P.nz;
    const int qrel = (int)blockIdx.x / CPJ;
    const int ybase = ((int)blockIdx.x - qrel * CPJ) * RG;
    const int qq = q0 + qrel;
    const int a = qq / nz, p = qq - a * nz;
    const bool pf = P.order >= 2;
    constexpr int np = NP;
    float zl[2], zh[2];  // z-boundary weights of this plane, per pole
    bool zb_any = false;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        zl[i] = (pf && i < np && p < ZPOW_N) ? P.tab.zpow[i * ZPOW_N + p] : 0.f;
        zh[i] = (pf && i < np && nz - 1 - p < ZPOW_N) ? P.tab.zpow[i * ZPOW_N + nz - 1 - p] : 0.f;
        zb_any = zb_any || zl[i] != 0.f || zh[i] != 0.f;
    }
    // slots of this thread in the all-zero column band
    unsigned zmask = 0;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int x = j + r * TPL;
        if (x >= P.kx_zero_lo && x < P.kx_zero_hi)
            zmask |= 1u << r;
    }
    // x-prefilter boundary weights of this thread's cropped slots for the
    // first pole: the A term (z^xx) for xx < ZPOW_N, the B term
    // (z^(NX-1-xx)) near the end
    float za[4], zb[4];
#pragma unroll
    for (int r = 2; r <= 5; ++r) {
        const int xx = j + TPL * (r - 2);
        za[r - 2] = (pf && xx < ZPOW_N) ? P.tab.zpow[xx] : 0.f;
        zb[r - 2] = (pf && NX - 1 - xx < ZPOW_N) ? P.tab.zpow[NX - 1 - xx] : 0.f;
    }
    const float2 *Tq = T + (size_t)qrel * NX * N + j;
    float2 *dst = slab + ((size_t)a * nz + p) * NX * NX + ybase;
    auto load_row = [&](int y, float2 (&v)[L::SLOTS]) {
        const float2 *src = Tq + (size_t)y * N;
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r)
            v[r] = (zmask >> r) & 1u ? make_float2(0.f, 0.f) : __ldcs(src + r * TPL);
    };
    // YD: the y-prefilter coefficient rows of this job, [2 NP][N] after the
    // edge slots (CTAs with boundary rows)
    float2 *ycs = edge + EDGE_SLOTS * LPC;
    const float2 *yed = T + P.yedge_off + (size_t)qrel * 4 * NP * N;
    if constexpr (YD && ycoef_smem<L>()) {
        if (ybase < ZPOW_N || ybase + RG - 1 >= NX - ZPOW_N) {
            for (int x = threadIdx.x; x < N; x += LPC * TPL) {
                float2 cy[2 * NP];
                if (!(x >= P.kx_zero_lo && x < P.kx_zero_hi)) {
                    float2 ed[EDGE_SLOTS];
#pragma unroll
                    for (int e = 0; e < EDGE_SLOTS; ++e)
                        ed[e] = edge_used(e, NP) ? yed[(size_t)edge_row(e, NP) * N + x] : make_float2(0.f, 0.f);
                    pf_coefs<NP>(P.kys, ed, cy);
                } else {
#pragma unroll
                    for (int i = 0; i < 2 * NP; ++i)
                        cy[i] = make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int i = 0; i < 2 * NP; ++i)
                    ycs[i * N + x] = cy[i];
            }
        }
    }
    float2 v[L::SLOTS], vn[L::SLOTS];
    load_row(ybase + l, v);
    __syncthreads();  // twiddles (and the coefficient rows)
#pragma unroll 1
    for (int g = 0; g < G; ++g) {
        const int y = ybase + g * LPC + l;
        if (g + 1 < G)
            load_row(y + LPC, vn);
        if constexpr (YD) {
            if (y < ZPOW_N || NX - 1 - y < ZPOW_N) {
#pragma unroll
                for (int r = 0; r < L::SLOTS; ++r) {
                    if (!((zmask >> r) & 1u)) {
                        const int x = j + r * TPL;
                        float2 cy[2 * NP];
                        if constexpr (ycoef_smem<L>()) {
#pragma unroll
                            for (int i = 0; i < 2 * NP; ++i)
                                cy[i] = ycs[i * N + x];
                        } else {
                            float2 ed[EDGE_SLOTS];
#pragma unroll
                            for (int e = 0; e < EDGE_SLOTS; ++e)
                                ed[e] = edge_used(e, NP) ? yed[(size_t)edge_row(e, NP) * N + x]
                                                         : make_float2(0.f, 0.f);
                            pf_coefs<NP>(P.kys, ed, cy);
                        }
                        v[r] = pf_apply<NP>(P, cy, y, NX, v[r]);
                    }
                }
            }
        }
        if (zb_any) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                if (i < np) {
                    const float2 *ta = Tab + ((size_t)(a * 2 * np + i) * NX + y) * N + j;
                    const float2 *tb = Tab + ((size_t)(a * 2 * np + np + i) * NX + y) * N + j;
#pragma unroll
                    for (int r = 0; r < L::SLOTS; ++r) {
                        if (!((zmask >> r) & 1u)) {
                            const float2 u = ta[r * TPL], w = tb[r * TPL];
                            v[r] = make_float2(fmaf(zh[i], w.x, fmaf(zl[i], u.x, v[r].x)),
                                               fmaf(zh[i], w.y, fmaf(zl[i], u.y, v[r].y)));
                        }
                    }
                }
            }
        }
        int flip = 0;
        line.template run<1>(v, j, buf0 + l * ls, buf1 + l * ls, 1, tw, flip, bar);
        if (pf) {
            // the samples around the crop's ends: each held by one thread,
            // at a compile-time slot
#pragma unroll
            for (int e = 0; e < EDGE_SLOTS; ++e) {
                float2 t;
                if (edge_used(e, np) && held<L>(v, j, PAD + edge_offset(e, NX), t))
                    edge[l * EDGE_SLOTS + e] = t;
            }
            line_sync(bar, TPL);
            float2 cf[2 * NP];
            pf_coefs<NP>(P.kxs, edge + l * EDGE_SLOTS, cf);
            const float2 Ac = cf[0], Bc = cf[np];  // first pole
#pragma unroll
            for (int r = 2; r <= 5; ++r) {
                v[r] = make_float2(fmaf(Bc.x, zb[r - 2], fmaf(Ac.x, za[r - 2], v[r].x)),
                                   fmaf(Bc.y, zb[r - 2], fmaf(Ac.y, za[r - 2], v[r].y)));
            }
            if constexpr (NP == 2) {  // second pole (orders 4, 5)
                const float2 A2 = cf[1], B2 = cf[3];
#pragma unroll
                for (int r = 2; r <= 5; ++r) {
                    const int xx = j + TPL * (r - 2);
                    if (xx < ZPOW_N) {
                        const float z = P.tab.zpow[ZPOW_N + xx];
                        v[r] = make_float2(fmaf(A2.x, z, v[r].x), fmaf(A2.y, z, v[r].y));
                    }
                    if (NX - 1 - xx < ZPOW_N) {
                        const float z = P.tab.zpow[ZPOW_N + NX - 1 - xx];
                        v[r] = make_float2(fmaf(B2.x, z, v[r].x), fmaf(B2.y, z, v[r].y));
                    }
                }
            }
        }
        // stage[x][l] (pitch LPC+1) in buf0, then runs of LPC y per x
        __syncthreads();  // every line is done with buf0 (and edge)
        float2 *stage = buf0;
        constexpr int SP = LPC + 1;
#pragma unroll
        for (int r = 2; r <= 5; ++r)
            stage[(j + TPL * (r - 2)) * SP + l] = v[r];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NX / TPL; ++k) {
            const int e = threadIdx.x + k * LPC * TPL;
            const int xx = e / LPC, ll = e % LPC;
            __stcs(dst + (size_t)xx * NX + g * LPC + ll, stage[xx * SP + ll]);
        }
        if (g + 1 < G) {
            __syncthreads();  // stage reads done before buf0 is reused
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r)
                v[r] = vn[r];
        }
    }
}

// (b1+b2) single-row planes (lNy == ny == 1, slab pitch 1: the 2D
// reconstruction): the column transforms are the identity, so a job's row
// is the row spectrum times the filter table (and gains) and the propagator
// of its plane, formed here instead of in a column stage.  A CTA takes RG
// consecutive jobs as groups of LPC lines (one job per line).  With one
// line per group the propagator is anchored exactly at the CTA's first job
// (and wherever the angle changes) and advanced plane by plane with the
// complex step exp(i w), as in k_columns_propagate; with several lines per
// group every line is anchored exactly.  Then per line the z-boundary rows
// of its plane, the backward FFT along x, the x-prefilter boundary terms,
// and the cropped row stored contiguously at slab[a][p][x].
template <class L, int LPC, int NP>
__global__ void __launch_bounds__(LPC * L::TPL, (LPC * L::TPL <= 256) ? 3 : 1)
    k_rows_line(StageParams P, L line, const float2 *rowspec, const float2 *Tab, float2 *slab, int q0, int qn)
{
    constexpr int RG = rows_per_cta<LPC>(), G = RG / LPC;
    extern __shared__ float2 smem[];
    const int n = line.size();  // lNx
    const int ls = xslots<false>(n);
    float2 *buf0 = smem, *buf1 = smem + LPC * ls, *tw = smem + 2 * LPC * ls;
    copy_twiddles<L>(tw, P.tab.twx, n);
    const int l = threadIdx.x / L::TPL, j = threadIdx.x % L::TPL;
    const int bar = (L::TPL % 32 == 0 && LPC < 15) ? 1 + l : 0;
    const int nx = P.nx, nz = P.nz, padxl = P.padxl;
    const bool pf = P.order >= 2;
    const int qbase = (int)blockIdx.x * RG;
    const int GV = min(G, (qn - qbase + LPC - 1) / LPC);  // groups holding a job
    float2 W[L::SLOTS];  // LPC == 1: the next plane's propagated spectrum
    int cur_a = -1;
    __syncthreads();  // twiddles
#pragma unroll 1
    for (int g = 0; g < GV; ++g) {
        const int qrel = qbase + g * LPC + l;
        const bool valid = qrel < qn;
        const int q = q0 + (valid ? qrel : 0);
        const int a = q / nz, p = q - a * nz;
        float2 v[L::SLOTS];
        if (LPC == 1 && a == cur_a) {
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int x = j + r * L::TPL;
                v[r] = W[r];
                if (column_active(P, x))
                    W[r] = cmul(W[r], P.tab.step[x]);
            }
        } else {
            const float zp = (float)p - 0.5f * (float)nz + P.zshift;
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int x = j + r * L::TPL;
                float2 b = make_float2(0.f, 0.f);
                if (valid && column_active(P, x)) {
                    b = cmul(rowspec[(size_t)a * n + x], P.tab.G[x]);
                    if (P.gain)
                        b = cscale(b, P.gain[x]);
                    if (P.again)
                        b = cmul(b, P.again[(size_t)a * n + x]);
                    b = cmul(b, expi_phase(P.tab.wsplit[x], zp));
                }
                v[r] = b;
                if (LPC == 1)
                    W[r] = column_active(P, x) ? cmul(b, P.tab.step[x]) : b;
            }
            cur_a = a;
        }
        if (valid && pf) {
            constexpr int np = NP;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const float zl = (i < np && p < ZPOW_N) ? P.tab.zpow[i * ZPOW_N + p] : 0.f;
                const float zh = (i < np && nz - 1 - p < ZPOW_N) ? P.tab.zpow[i * ZPOW_N + nz - 1 - p] : 0.f;
                if (zl != 0.f || zh != 0.f) {
                    const float2 *ta = Tab + (size_t)(a * 2 * np + i) * n;
                    const float2 *tb = Tab + (size_t)(a * 2 * np + np + i) * n;
#pragma unroll
                    for (int r = 0; r < L::SLOTS; ++r) {
                        const int x = j + r * L::TPL;
                        if (column_active(P, x)) {
                            const float2 u = ta[x], w = tb[x];
                            v[r] = make_float2(fmaf(zh, w.x, fmaf(zl, u.x, v[r].x)),
                                               fmaf(zh, w.y, fmaf(zl, u.y, v[r].y)));
                        }
                    }
                }
            }
        }
        int flip = 0;
        line.template run<1>(v, j, buf0 + l * ls, buf1 + l * ls, 1, tw, flip, bar);
        float2 cf[2 * NP];
        if (pf) {
            // the line's samples at x0-1, x0+1, x1-1, x1+1 (periodic), through
            // the exchange buffer the FFT's last exchange did not use
            float2 *sc = (flip ? buf1 : buf0) + l * ls;
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int x = j + r * L::TPL;
                if (x < n)
                    sc[x] = v[r];
            }
            if (bar > 0)
                line_sync(bar, L::TPL);
            else
                __syncthreads();
            float2 ed[EDGE_SLOTS];
#pragma unroll
            for (int e = 0; e < EDGE_SLOTS; ++e)
                ed[e] = edge_used(e, NP) ? sc[(padxl + edge_offset(e, nx) + 2 * n) % n] : make_float2(0.f, 0.f);
            pf_coefs<NP>(P.kxs, ed, cf);
        }
        if (valid) {
            float2 *dst = slab + ((size_t)a * nz + p) * nx;
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int xx = j + r * L::TPL - padxl;
                if (xx >= 0 && xx < nx) {
                    float2 o = v[r];
                    if (pf)
                        o = pf_apply<NP>(P, cf, xx, nx, o);
                    __stcs(dst + xx, o);
                }
            }
        }
        // the edge reads of this group end before the next group's FFT
        // writes the exchange buffers
        if (g + 1 < GV) {
            if (bar > 0)
                line_sync(bar, L::TPL);
            else
                __syncthreads();
        }
    }
}

// (b0) z-prefilter boundary columns for single-row planes: the column
// transforms are the identity, Tab[a][t][kx] = spectrum * G * (alpha, beta).
__global__ void __launch_bounds__(256) k_columns_boundary_line(StageParams P, const float2 *rowspec, float2 *Tab,
                                                               int nb)
{
    const int lNx = P.lNx;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nb * lNx)
        return;
    const int a = (int)(i / lNx), kx = (int)(i - (long long)a * lNx);
    float2 b = make_float2(0.f, 0.f);
    if (column_active(P, kx)) {
        b = cmul(rowspec[(size_t)a * lNx + kx], P.tab.G[kx]);
        if (P.gain)
            b = cscale(b, P.gain[kx]);
        if (P.again)
            b = cmul(b, P.again[(size_t)a * lNx + kx]);
    }
    const int np = P.npoles;
    const size_t K = (size_t)P.lNy * lNx;
    for (int i = 0; i < np; ++i) {
        Tab[(size_t)(a * 2 * np + i) * lNx + kx] = cmul(b, P.tab.alpha[i * K + kx]);
        Tab[(size_t)(a * 2 * np + np + i) * lNx + kx] = cmul(b, P.tab.beta[i * K + kx]);
    }
}

// ---------------------------------------------------------------------------
// Planes per column-stage CTA: enough CTAs for one full wave of the
// resident slots over the active column groups (the forward column FFT of a
// CTA is amortised over its planes, so fewer, longer CTAs are better as long
// as every slot is busy), at least 4 and at most 256 for long runs
// (long_runs), else at most kReanchorPlanes.
template <int KX>
static int planes_per_cta(const StageParams &P, int qn, bool long_run)
{
    const int groups = (P.lNx + KX - 1) / KX;
    int active = 0;
    for (int g = 0; g < groups; ++g)
        if (!(g * KX >= P.kx_zero_lo && g * KX + KX <= P.kx_zero_hi))
            ++active;
    const int per = P.col_slots > 0 ? std::max(1, P.col_slots / std::max(1, active)) : 4;
    const int ppc = (qn + per - 1) / per;
    return std::min(long_run ? 256 : kReanchorPlanes, std::max(4, ppc));
}

// Shared memory of the generic-crop column kernel: power-of-two columns of
// 512 or more carry the third-pass twiddle table and the filtered-spectrum
// region as the half-crop kernel does.
template <class L>
static size_t smem_cols_prop(int n)
{
    return (column_regs<L, Cfg<L>::KX, false>() && pow2_len<L>() >= 512) ? smem_cols_half<L>(n) : smem_cols<L>(n);
}

// Calls fn(std::integral_constant<int, V>) for V = v (one of 0, 1, 2), so a
// pole count chosen at run time selects a compile-time instantiation.
template <class F>
static cudaError_t with_poles(int v, F &&fn)
{
    switch (v) {
    case 0: return fn(std::integral_constant<int, 0>{});
    case 1: return fn(std::integral_constant<int, 1>{});
    case 2: return fn(std::integral_constant<int, 2>{});
    default: return cudaErrorInvalidValue;
    }
}
// Poles of the y-prefilter the column stage applies (tilted path, order
// >= 2), 0 for none; poles of the x- and z-prefilters of the row stages
// (1 also for orders 0 and 1, where the row stages skip the prefilter).
static int column_poles(const StageParams &P)
{
    return (P.tilted && P.order >= 2) ? P.npoles : 0;
}
static int row_poles(const StageParams &P)
{
    return P.order >= 4 ? 2 : 1;
}

template <class L>
static cudaError_t rows_forward_impl(const StageParams &P, L line, const void *sino, const double *w, int nb,
                                     float2 *out, cudaStream_t s)
{
    constexpr int LPC = Cfg<L>::LPC;
    const long long lines = (long long)nb * P.lNy;
    const unsigned grid = (unsigned)((lines + LPC - 1) / LPC);
    k_rows_forward<L, LPC><<<grid, LPC * L::TPL, smem_rows<L>(line.n), s>>>(P, line, sino, w, nb, out);
    return cudaGetLastError();
}

template <class L>
static cudaError_t boundary_impl(const StageParams &P, L line, const float2 *rowspec, float2 *Tab, int nb,
                                 cudaStream_t s)
{
    constexpr int KX = Cfg<L>::KX;
    dim3 grid((P.lNx + KX - 1) / KX, nb);
    return with_poles(column_poles(P), [&](auto yf) {
        k_columns_boundary<L, KX, decltype(yf)::value>
            <<<grid, KX * L::TPL, smem_cols<L>(line.n), s>>>(P, line, rowspec, Tab);
        return cudaGetLastError();
    });
}

// Lines of a half-crop row kernel: whole warps (the line barriers are
// per line).
template <class L>
constexpr bool half_line()
{
    return pow2_len<L>() >= 256;
}
// Groups of lines per half-crop row CTA (LPC * G rows): 16 rows, so that
// the CTA's set-up (twiddle table, boundary weights, zero-column mask) is
// shared by more lines (256^3 workload: 8 rows 21.7 ms, 16 rows 20.9 ms,
// 32 rows 21.2 ms for the row stage).
template <class L>
constexpr int half_groups()
{
    return Cfg<L>::LPC >= 16 ? 1 : 16 / Cfg<L>::LPC;
}
template <class L>
static cudaError_t columns_impl(const StageParams &P, L line, const float2 *rowspec, float2 *T, int q0, int qn,
                                cudaStream_t s)
{
    constexpr int KX = Cfg<L>::KX;
    bool half = false;
    if constexpr (half_line<L>())
        half = half_crop(P);
    const int ppc = planes_per_cta<KX>(P, qn, half ? long_runs<L, KX, true>() : long_runs<L, KX, false>());
    dim3 grid((P.lNx + KX - 1) / KX, (qn + ppc - 1) / ppc);
    return with_poles(column_poles(P), [&](auto yf) {
        constexpr int YF = decltype(yf)::value;
        if constexpr (half_line<L>()) {
            if (half_crop(P)) {
                k_columns_propagate<L, KX, true, YF>
                    <<<grid, KX * L::TPL, smem_cols_half<L>(line.n), s>>>(P, line, rowspec, T, q0, qn, ppc);
                return cudaGetLastError();
            }
        }
        k_columns_propagate<L, KX, false, YF>
            <<<grid, KX * L::TPL, smem_cols_prop<L>(line.n), s>>>(P, line, rowspec, T, q0, qn, ppc);
        return cudaGetLastError();
    });
}

template <class L>
static cudaError_t rows_inverse_impl(const StageParams &P, L line, const float2 *T, const float2 *Tab,
                                     float2 *slab, int q0, int qn, cudaStream_t s)
{
    constexpr int LPC = Cfg<L>::LPC;
    return with_poles(row_poles(P), [&](auto np) {
        constexpr int NP = decltype(np)::value;
        if constexpr (NP >= 1) {
            if constexpr (half_line<L>()) {
                if (half_crop(P)) {
                    constexpr int G = half_groups<L>();
                    const unsigned grid = (unsigned)((long long)qn * (L::N / 2 / (LPC * G)));
                    if (P.ydefer)
                        k_rows_inverse_half<L, LPC, G, NP, true>
                            <<<grid, LPC * L::TPL, smem_rows_half<L>(line.n) + smem_rows_y<L, NP, true>(line.n),
                               s>>>(P, line, T, Tab, slab, q0);
                    else
                        k_rows_inverse_half<L, LPC, G, NP, false>
                            <<<grid, LPC * L::TPL, smem_rows_half<L>(line.n), s>>>(P, line, T, Tab, slab, q0);
                    return cudaGetLastError();
                }
            }
            const unsigned grid =
                (unsigned)((long long)qn * ((P.ny + rows_per_cta<LPC>() - 1) / rows_per_cta<LPC>()));
            if (P.ydefer)
                k_rows_inverse<L, LPC, NP, true>
                    <<<grid, LPC * L::TPL, smem_rows<L>(line.n) + smem_rows_y<L, NP, true>(line.n), s>>>(
                        P, line, T, Tab, slab, q0, qn);
            else
                k_rows_inverse<L, LPC, NP, false>
                    <<<grid, LPC * L::TPL, smem_rows<L>(line.n), s>>>(P, line, T, Tab, slab, q0, qn);
            return cudaGetLastError();
        } else {
            return cudaErrorInvalidValue;
        }
    });
}

// The attribute is per kernel and process-wide, so it is always set to the
// largest size the instantiation can need (the generic line serves every
// length up to its maximum).
template <class L, int NP>
static cudaError_t set_smem_attrs_np(int n)
{
    cudaError_t e;
    if constexpr (NP >= 1) {
        e = cudaFuncSetAttribute(k_rows_inverse<L, Cfg<L>::LPC, NP, false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_rows<L>(n));
        if (e != cudaSuccess)
            return e;
        e = cudaFuncSetAttribute(k_rows_inverse<L, Cfg<L>::LPC, NP, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(smem_rows<L>(n) + smem_rows_y<L, NP, true>(n)));
        if (e != cudaSuccess)
            return e;
        e = cudaFuncSetAttribute(k_rows_line<L, Cfg<L>::LPC, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem_rows<L>(n));
        if (e != cudaSuccess)
            return e;
    }
    if constexpr (half_line<L>()) {
        e = cudaFuncSetAttribute(k_columns_propagate<L, Cfg<L>::KX, true, NP>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cols_half<L>(n));
        if (e != cudaSuccess)
            return e;
        if constexpr (NP >= 1) {
            e = cudaFuncSetAttribute(k_rows_inverse_half<L, Cfg<L>::LPC, half_groups<L>(), NP, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_rows_half<L>(n));
            if (e != cudaSuccess)
                return e;
            e = cudaFuncSetAttribute(k_rows_inverse_half<L, Cfg<L>::LPC, half_groups<L>(), NP, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(smem_rows_half<L>(n) + smem_rows_y<L, NP, true>(n)));
            if (e != cudaSuccess)
                return e;
        }
    }
    e = cudaFuncSetAttribute(k_columns_boundary<L, Cfg<L>::KX, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_cols<L>(n));
    if (e != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_columns_propagate<L, Cfg<L>::KX, false, NP>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cols_prop<L>(n));
}

template <class L>
static cudaError_t set_smem_attrs(int n)
{
    if (std::is_same<L, GenericLine>::value)
        n = GenericLine::TPL * GenericLine::SLOTS;
    cudaError_t e;
    e = cudaFuncSetAttribute(k_rows_forward<L, Cfg<L>::LPC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_rows<L>(n));
    if (e != cudaSuccess)
        return e;
    for (int np = 0; np <= 2; ++np) {
        e = with_poles(np, [&](auto v) { return set_smem_attrs_np<L, decltype(v)::value>(n); });
        if (e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

int columns_slots(const StageParams &P)
{
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    const cudaError_t e = with_line(P.lNy, [&](auto line) {
        using L = decltype(line);
        constexpr int KX = Cfg<L>::KX;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_columns_propagate<L, KX, false, 0>,
                                                             KX * L::TPL, smem_cols_prop<L>(line.n));
    });
    return e == cudaSuccess ? per * sms : 0;
}

bool line_size_supported(int n)
{
    switch (n) {
    case 64: case 128: case 256: case 512: case 1024: case 2048: case 4096: return true;
    default: return n >= 1 && n <= GenericLine::TPL * GenericLine::SLOTS;
    }
}

cudaError_t configure_kernels(const StageParams &P)
{
    cudaError_t e = with_line(P.lNx, [&](auto line) { return set_smem_attrs<decltype(line)>(line.n); });
    if (e != cudaSuccess)
        return e;
    return with_line(P.lNy, [&](auto line) { return set_smem_attrs<decltype(line)>(line.n); });
}

cudaError_t launch_rows_forward(const StageParams &P, const void *sino_batch, const double *weights_batch, int nb,
                                float2 *rowspec, cudaStream_t s)
{
    return with_line(P.lNx, [&](auto line) {
        return rows_forward_impl(P, line, sino_batch, weights_batch, nb, rowspec, s);
    });
}

cudaError_t launch_columns_propagate(const StageParams &P, const float2 *rowspec, float2 *T, int q0, int qn,
                                     cudaStream_t s)
{
    return with_line(P.lNy, [&](auto line) { return columns_impl(P, line, rowspec, T, q0, qn, s); });
}

bool half_crop(const StageParams &P)
{
    const int N = P.lNx;
    return P.lNy == N && N >= 256 && N <= 4096 && (N & (N - 1)) == 0 && 2 * P.ny == N && 2 * P.nx == N &&
           4 * P.padyl == N && 4 * P.padxl == N && P.nz == P.nx && P.ypitch == P.ny;
}

bool single_row_plan(const StageParams &P)
{
    return P.lNy == 1 && P.ny == 1 && P.padyl == 0 && P.ypitch == 1;
}

cudaError_t launch_rows_line(const StageParams &P, const float2 *rowspec, const float2 *Tab, float2 *slab, int q0,
                             int qn, cudaStream_t s)
{
    return with_line(P.lNx, [&](auto line) {
        using L = decltype(line);
        constexpr int LPC = Cfg<L>::LPC;
        const unsigned grid = (unsigned)((qn + rows_per_cta<LPC>() - 1) / rows_per_cta<LPC>());
        return with_poles(row_poles(P), [&](auto np) {
            constexpr int NP = decltype(np)::value;
            if constexpr (NP >= 1) {
                k_rows_line<L, LPC, NP>
                    <<<grid, LPC * L::TPL, smem_rows<L>(line.n), s>>>(P, line, rowspec, Tab, slab, q0, qn);
                return cudaGetLastError();
            } else {
                return cudaErrorInvalidValue;
            }
        });
    });
}

cudaError_t launch_columns_boundary(const StageParams &P, const float2 *rowspec, float2 *Tab, int nb,
                                    cudaStream_t s)
{
    if (single_row_plan(P)) {
        const long long n = (long long)nb * P.lNx;
        k_columns_boundary_line<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, rowspec, Tab, nb);
        return cudaGetLastError();
    }
    return with_line(P.lNy, [&](auto line) { return boundary_impl(P, line, rowspec, Tab, nb, s); });
}

cudaError_t launch_rows_inverse(const StageParams &P, const float2 *T, const float2 *Tab, float2 *slab, int q0,
                                int qn, cudaStream_t s)
{
    return with_line(P.lNx, [&](auto line) { return rows_inverse_impl(P, line, T, Tab, slab, q0, qn, s); });
}

}  // namespace odt
