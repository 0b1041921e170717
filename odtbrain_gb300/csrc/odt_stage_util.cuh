// Device helpers and launch-shape policy shared by the filter stages
// (stages.cu) and their adjoints (adjoint.cu).
#pragma once
#include <type_traits>

#include "odt_fft.cuh"
#include "odt_internal.cuh"

namespace odt {

// exp(i * w * z) with w held as (hi, lo) floats and z a small half-integer:
// exact product hi*z via FMA, Cody-Waite reduction by 2*pi, then sincosf.
__device__ __forceinline__ float2 expi_phase(float2 w, float z)
{
    const float ph = w.x * z;
    const float err = fmaf(w.x, z, -ph);
    const float lo = fmaf(w.y, z, err);
    const float k = rintf(ph * 0.15915494309189535f);
    float r = fmaf(-k, 6.28125f, ph);
    r = fmaf(-k, 1.9353071795864769253e-3f, r);
    r += lo;
    float s, c;
    sincosf(r, &s, &c);
    return make_float2(c, s);
}

__device__ __forceinline__ float2 load_sino(const void *sino, int in_c128, size_t idx, double w)
{
    if (in_c128) {
        const double2 v = reinterpret_cast<const double2 *>(sino)[idx];
        return make_float2((float)(v.x * w), (float)(v.y * w));
    }
    const float2 v = reinterpret_cast<const float2 *>(sino)[idx];
    const float wf = (float)w;
    return make_float2(v.x * wf, v.y * wf);
}

// np.pad linear_ramp value at ramp position i of `width` (i = 0 is the
// outer edge): end + (edge - end) * i / width  (numpy linspace, endpoint
// False).
__device__ __forceinline__ float2 ramp(float2 edge, float2 end, int i, int width)
{
    const float t = (float)i / (float)width;
    return make_float2(fmaf(edge.x - end.x, t, end.x), fmaf(edge.y - end.y, t, end.y));
}

// Padded, weighted sample (y, x) of the padded plane of angle row `arow`
// (odtbrain/_alg3d_bpp.py:493-506: np.pad pads y first, then x).
__device__ __forceinline__ float2 padded_sample(const StageParams &P, const void *sino, size_t arow, double w, int y, int x)
{
    const int ny = P.ny, nx = P.nx;
    if (P.pad_mode == 0)
        return load_sino(sino, P.in_c128, arow + (size_t)y * nx + x, w);
    const int ys = y - P.padyl, xs = x - P.padxl;
    if (P.pad_mode == 1) {
        const int yc = min(max(ys, 0), ny - 1), xc = min(max(xs, 0), nx - 1);
        return load_sino(sino, P.in_c128, arow + (size_t)yc * nx + xc, w);
    }
    const int padyr = P.lNy - ny - P.padyl, padxr = P.lNx - nx - P.padxl;
    auto colval = [&](int xc) -> float2 {
        if (ys >= 0 && ys < ny)
            return load_sino(sino, P.in_c128, arow + (size_t)ys * nx + xc, w);
        if (ys < 0)
            return ramp(load_sino(sino, P.in_c128, arow + xc, w), P.padval, y, P.padyl);
        const int jdx = ys - ny;
        return ramp(load_sino(sino, P.in_c128, arow + (size_t)(ny - 1) * nx + xc, w), P.padval,
                    padyr - 1 - jdx, padyr);
    };
    if (xs >= 0 && xs < nx)
        return colval(xs);
    if (xs < 0)
        return ramp(colval(0), P.padval, x, P.padxl);
    return ramp(colval(nx - 1), P.padval, padxr - 1 - (xs - nx), padxr);
}

// ---------------------------------------------------------------------------
// Prefilter boundary terms of a cropped line (see the filter stages' header
// comment).  The transform's output u is the particular solution; the line
// of n samples starting at `pad` gets c[k] = u[pad+k] + sum_i A_i z_i^k +
// B_i z_i^(n-1-k), with (A_1.., B_1..) = K (d_1L.., d_1R..) and d_mL =
// u[m] - u[-m], d_mR = u[n-1-m] - u[n-1+m] (indices relative to pad).
// Edge samples, relative to pad: slot 2q, 2q+1 hold u[-(q+1)], u[q+1]
// (q < npoles) and slot 4+2q, 4+2q+1 hold u[n-2-q], u[n+q].
__host__ __device__ constexpr int edge_offset(int slot, int n)
{
    return slot < 4 ? ((slot & 1) ? 1 + (slot >> 1) : -(1 + (slot >> 1)))
                    : ((slot & 1) ? n + ((slot - 4) >> 1) : n - 2 - ((slot - 4) >> 1));
}
constexpr int EDGE_SLOTS = 8;
// True for the slots a prefilter of np poles reads (q < np).
__host__ __device__ constexpr bool edge_used(int slot, int np)
{
    return ((slot & 3) >> 1) < np;
}
// Row of a used edge slot among the 4 np rows of the deferred y-prefilter's
// edge samples (the slots at the crop's start, then those at its end).
__host__ __device__ constexpr int edge_row(int slot, int np)
{
    return slot < 4 ? slot : 2 * np + (slot - 4);
}

// Coefficients of an NP-pole prefilter (NP = 1: orders 2, 3; NP = 2:
// orders 4, 5) from the edge slots: c[i] = A_(i+1), c[NP + i] = B_(i+1).
// K is the 2NP x 2NP boundary solve, row-major.  NP is a compile-time
// constant so that c stays in registers.
template <int NP>
__device__ __forceinline__ void pf_coefs(const float *K, const float2 *ed, float2 (&c)[2 * NP])
{
    float2 d[2 * NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        d[q] = ed[2 * q + 1] - ed[2 * q];               // u[q+1] - u[-(q+1)]
        d[NP + q] = ed[4 + 2 * q] - ed[4 + 2 * q + 1];  // u[n-2-q] - u[n+q]
    }
#pragma unroll
    for (int r = 0; r < 2 * NP; ++r) {
        c[r] = make_float2(0.f, 0.f);
#pragma unroll
        for (int jj = 0; jj < 2 * NP; ++jj) {
            const float k = K[r * 2 * NP + jj];
            c[r] = make_float2(fmaf(k, d[jj].x, c[r].x), fmaf(k, d[jj].y, c[r].y));
        }
    }
}

// Output k of the n-sample line with its boundary terms added.
template <int NP>
__device__ __forceinline__ float2 pf_apply(const StageParams &P, const float2 (&c)[2 * NP], int k, int n, float2 o)
{
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        if (k < ZPOW_N) {
            const float z = P.tab.zpow[i * ZPOW_N + k];
            o = make_float2(fmaf(c[i].x, z, o.x), fmaf(c[i].y, z, o.y));
        }
        if (n - 1 - k < ZPOW_N) {
            const float z = P.tab.zpow[i * ZPOW_N + n - 1 - k];
            o = make_float2(fmaf(c[NP + i].x, z, o.x), fmaf(c[NP + i].y, z, o.y));
        }
    }
    return o;
}

// The twiddle region (tw_slots(n) entries) from the plain table `src`.
template <class L>
__device__ __forceinline__ void copy_twiddles(float2 *dst, const float2 *src, int n)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        dst[i] = src[i];
    if (!std::is_same<L, GenericLine>::value) {
        for (int i = threadIdx.x; i < TW_P1; i += blockDim.x) {
            const int jm = i / 7, r = i - 7 * jm + 1;
            dst[n + i] = src[r * jm * (n / 64)];
        }
    }
}


// copy_twiddles plus the third-pass table (tw_slots2(n) entries; power-of-
// two lines with a third radix-8 pass, n >= 512).
template <class L>
__device__ __forceinline__ void copy_twiddles2(float2 *dst, const float2 *src, int n)
{
    copy_twiddles<L>(dst, src, n);
    for (int i = threadIdx.x; i < TW_P2; i += blockDim.x) {
        const int jm = i / 7, r = i - 7 * jm + 1;
        dst[n + TW_P1 + i] = src[r * jm * (n / 512)];
    }
}

// Select v[pos / TPL] of the thread holding position `pos` without dynamic
// register indexing; returns true when this thread holds it.
template <class L>
__device__ __forceinline__ bool held(const float2 (&v)[L::SLOTS], int j, int pos, float2 &out)
{
    if (pos % L::TPL != j)
        return false;
    const int rr = pos / L::TPL;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r)
        if (r == rr)
            out = v[r];
    return true;
}

// True when spectrum column kx can be nonzero.
__device__ __forceinline__ bool column_active(const StageParams &P, int kx)
{
    return kx < P.lNx && (kx < P.kx_zero_lo || kx >= P.kx_zero_hi);
}

// True when any of the KX columns starting at kx0 can be nonzero.
template <int KX>
__device__ __forceinline__ bool group_active(const StageParams &P, int kx0)
{
    return !(kx0 >= P.kx_zero_lo && kx0 + KX <= P.kx_zero_hi);
}

// Length of a power-of-two line type, 0 for the generic line.
template <class L>
constexpr int pow2_len()
{
    if constexpr (std::is_same<L, GenericLine>::value)
        return 0;
    else
        return L::N;
}

// ---------------------------------------------------------------------------
// Dispatch on the line length.
// KX columns per column-stage CTA: 512-point columns run 4 per CTA (256
// threads) so that three CTAs of 85 registers fit an SM; measured on the
// 256^3 workload, 8 per CTA at 64 registers took 27.1 ms for the column
// stage against 25.7 ms (and 4 per CTA at 2 CTAs of 128 registers 28.7 ms).
template <class L>
struct Cfg {
    static constexpr int LPC = (L::TPL >= 256) ? 1 : 256 / L::TPL;
    static constexpr int KX = (L::TPL == 64) ? 4 : ((L::TPL >= 512) ? 1 : ((512 / L::TPL) > 16 ? 16 : 512 / L::TPL));
};
template <>
struct Cfg<GenericLine> {
    static constexpr int LPC = 4;
    static constexpr int KX = 4;
};

template <class L>
inline size_t smem_rows(int n)
{
    return (size_t)(2 * Cfg<L>::LPC * xslots<false>(n) + tw_slots(n) + EDGE_SLOTS * Cfg<L>::LPC) * sizeof(float2);
}
// k_rows_inverse_half: the exchange buffers, the twiddle table and the
// edge samples.
template <class L>
inline size_t smem_rows_half(int n)
{
    return (size_t)(2 * Cfg<L>::LPC * xslots<false>(n) + tw_slots(n) + EDGE_SLOTS * Cfg<L>::LPC) * sizeof(float2);
}
// k_columns_propagate of half-crop plans: smem_cols plus the third-pass
// twiddle table.
template <class L>
inline size_t smem_cols_half(int n)
{
    return (size_t)(2 * Cfg<L>::KX * xslots<true>(n) + Cfg<L>::KX * n + tw_slots2(n) + EDGE_SLOTS * Cfg<L>::KX) *
           sizeof(float2);
}
template <class L>
inline size_t smem_cols(int n)
{
    return (size_t)(2 * Cfg<L>::KX * xslots<true>(n) + Cfg<L>::KX * n + tw_slots(n) + EDGE_SLOTS * Cfg<L>::KX) *
           sizeof(float2);
}

// Calls fn(line) with the line type for length n.
template <class F>
inline cudaError_t with_line(int n, F &&fn)
{
    switch (n) {
    case 64: return fn(Pow2Line<64>{64});
    case 128: return fn(Pow2Line<128>{128});
    case 256: return fn(Pow2Line<256>{256});
    case 512: return fn(Pow2Line<512>{512});
    case 1024: return fn(Pow2Line<1024>{1024});
    case 2048: return fn(Pow2Line<2048>{2048});
    case 4096: return fn(Pow2Line<4096>{4096});
    default:
        if (n >= 1 && n <= GenericLine::TPL * GenericLine::SLOTS)
            return fn(GenericLine{n});
        return cudaErrorInvalidValue;
    }
}

}  // namespace odt
