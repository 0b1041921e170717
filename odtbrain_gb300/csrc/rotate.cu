// Stage (c) of the 3D backpropagation: B-spline resampling of every angle's
// coefficient slab and compensated accumulation into the volume.
//
// Reference: odtbrain/_alg3d_bpp.py:532-546 (scipy.ndimage.rotate of each
// (z, x) plane about y, real and imaginary parts, "+=" into the volume) and
// odtbrain/_alg3d_bppt.py:904-944 (scipy.ndimage.affine_transform of the
// (x, -y, z) volume).  The slabs arrive already prefiltered (the filter
// stages fold the spline prefilter in), so this stage only interpolates.
//
// scipy semantics reproduced (mode="constant", cval=0):
//   * coordinate i = ((off_i + m_i0*o_0) + m_i1*o_1) [+ m_i2*o_2] in FP64;
//     any coordinate outside [0, n-1] gives 0;
//   * taps that fall outside [0, n-1] read mirror-extended coefficients;
//   * tap start floor(c + 1/2) - order/2 (even order), floor(c) - order/2
//     (odd order), centred B-spline weights.
// Coordinates are evaluated in FP32 relative to an FP64 tile origin; a
// coordinate within 1e-3 of the domain boundary is re-evaluated in FP64 in
// the reference's operation order, so in/out decisions match the FP64
// oracle bit for bit.  Across angles the sum is Kahan-compensated in
// registers; across launches (angle batches) the compensation is carried in
// a side buffer.
#include <float.h>
#include "odt_fft.cuh"
#include "odt_internal.cuh"

namespace odt {

constexpr float kGuard = 1e-3f;

__device__ __forceinline__ int mirror_idx(int i, int n)
{
    if (n == 1)
        return 0;
    while (i < 0 || i > n - 1) {
        if (i < 0)
            i = -i;
        if (i > n - 1)
            i = 2 * (n - 1) - i;
    }
    return i;
}

template <int ORDER>
struct Spline;
template <>
struct Spline<0> {
    __device__ static int weights(float c, float *w)
    {
        w[0] = 1.f;
        return (int)floorf(c + 0.5f);
    }
};
template <>
struct Spline<1> {
    __device__ static int weights(float c, float *w)
    {
        const float s = floorf(c);
        const float t = c - s;
        w[0] = 1.f - t;
        w[1] = t;
        return (int)s;
    }
};
template <>
struct Spline<2> {
    __device__ static int weights(float c, float *w)
    {
        const float s = floorf(c + 0.5f);
        const float t = c - s;
        const float a = 0.5f - t, b = 0.5f + t;
        w[0] = 0.5f * a * a;
        w[1] = 0.75f - t * t;
        w[2] = 0.5f * b * b;
        return (int)s - 1;
    }
};
template <>
struct Spline<3> {
    __device__ static int weights(float c, float *w)
    {
        const float s = floorf(c);
        const float t = c - s;
        const float u = 1.f - t, t2 = t * t;
        w[0] = u * u * u * (1.f / 6.f);
        w[1] = (4.f - 6.f * t2 + 3.f * t2 * t) * (1.f / 6.f);
        w[2] = (1.f + 3.f * t + 3.f * t2 - 3.f * t2 * t) * (1.f / 6.f);
        w[3] = t2 * t * (1.f / 6.f);
        return (int)s - 1;
    }
};

// First tap index for an FP64 coordinate (used for footprints).
template <int ORDER>
__device__ __forceinline__ long long tap_start_d(double c)
{
    return (ORDER & 1) ? (long long)floor(c) - ORDER / 2 : (long long)floor(c + 0.5) - ORDER / 2;
}

// In/out decision for one axis.  `l` is the FP32 coordinate relative to the
// integer I (true coordinate ~ I + l); `exact` evaluates the FP64 coordinate
// in the reference's order when the FP32 estimate is too close to call.
template <class F>
__device__ __forceinline__ bool inside_axis(float l, int I, int n, F exact)
{
    const float lo = (float)(-I), hi = (float)(n - 1 - I);
    if (l > lo + kGuard && l < hi - kGuard)
        return true;
    if (l < lo - kGuard || l > hi + kGuard)
        return false;
    const double c = exact();
    return c >= 0.0 && c <= (double)(n - 1);
}

// A coordinate axis of a tile: c(d) = I + f + m0*d0 + m1*d1 for small
// integer offsets d of an output voxel from the tile origin.  Each slope is
// split as m = mh + ml with mh on a 2^-12 grid, so mh*d and their sum are
// exact in FP32 (|d| < 2^8) and only the tiny ml*d terms round; the result
// is returned as an integer base plus a fraction-sized float, accurate to
// ~1e-7 of a voxel.
struct AxisCoord {
    float f, mh0, ml0, mh1, ml1;
    int I;
};

__device__ __forceinline__ AxisCoord make_axis(double c0, double m0, double m1)
{
    AxisCoord a;
    const double I = floor(c0);
    a.I = (int)I;
    a.f = (float)(c0 - I);
    const double h0 = rint(m0 * 4096.0) / 4096.0, h1 = rint(m1 * 4096.0) / 4096.0;
    a.mh0 = (float)h0;
    a.ml0 = (float)(m0 - h0);
    a.mh1 = (float)h1;
    a.ml1 = (float)(m1 - h1);
    return a;
}

// Returns the fraction-sized part t and sets B so that c = B + t.
__device__ __forceinline__ float eval_axis(const AxisCoord &a, float d0, float d1, int &B)
{
    const float S = fmaf(a.mh1, d1, a.mh0 * d0);    // exact
    const float R = fmaf(a.ml1, d1, fmaf(a.ml0, d0, a.f));
    const float Sf = floorf(S);
    B = a.I + (int)Sf;
    return (S - Sf) + R;
}

__device__ __forceinline__ void kahan_add(float2 &s, float2 &c, float2 v)
{
    float y = v.x - c.x;
    float t = s.x + y;
    c.x = (t - s.x) - y;
    s.x = t;
    y = v.y - c.y;
    t = s.y + y;
    c.y = (t - s.y) - y;
    s.y = t;
}

// Store the compensated partial sum of this launch (s, c) for voxel `idx`.
template <bool ONLYREAL>
__device__ __forceinline__ void store_sum(const RotParams &R, void *volume, float2 *comp, size_t idx, float2 s,
                                          float2 c)
{
    float2 S, C;
    if (R.first_pass) {
        S = s;
        C = c;
    } else {
        float2 S1, C1 = comp[idx];
        if (ONLYREAL)
            S1 = make_float2(reinterpret_cast<float *>(volume)[idx], 0.f);
        else
            S1 = reinterpret_cast<float2 *>(volume)[idx];
        // (S1 - C1) + (s - c), compensated
        float y = (s.x - c.x) - C1.x;
        float t = S1.x + y;
        C.x = (t - S1.x) - y;
        S.x = t;
        y = (s.y - c.y) - C1.y;
        t = S1.y + y;
        C.y = (t - S1.y) - y;
        S.y = t;
    }
    if (R.last_pass) {
        S = make_float2(S.x - C.x, S.y - C.y);
    } else {
        comp[idx] = C;
    }
    if (ONLYREAL)
        reinterpret_cast<float *>(volume)[idx] = S.x;
    else
        reinterpret_cast<float2 *>(volume)[idx] = S;
}

// ---------------------------------------------------------------------------
// y-axis path: every (z, x) plane at fixed y is rotated; the slab layout is
// [a][y][z][x] so that a plane is contiguous.
constexpr int RY_T = 32;       // output tile is 32 (z) x 32 (x)
constexpr int RY_BOX = 52;     // footprint of a rotated tile + taps + margin
constexpr int RY_BP = 53;      // shared-memory row pitch (float2)

template <int ORDER, bool ONLYREAL>
__global__ void __launch_bounds__(256) k_rotate_y(RotParams R, const float2 *__restrict__ slab,
                                                  const double *__restrict__ geo, void *volume, float2 *comp)
{
    __shared__ float2 box[RY_BOX * RY_BP];
    __shared__ double sg[6];
    __shared__ AxisCoord sax[2];  // z, x coordinates at the tile origin
    __shared__ int si[4];         // box z0, box x0, box nz (<=0: skip), box nx
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int ox0 = blockIdx.x * RY_T, oz0 = blockIdx.y * RY_T, y = blockIdx.z;
    const int nx = R.nx, nz = R.nz, ny = R.ny;
    const int ox = ox0 + tx;
    float2 s[4], cp[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        s[q] = make_float2(0.f, 0.f);
        cp[q] = make_float2(0.f, 0.f);
    }
    for (int a = 0; a < R.nbatch_angles; ++a) {
        if (threadIdx.x == 0) {
            const double *g = geo + 6 * (size_t)a;
            const double m00 = g[0], m01 = g[1], m10 = g[2], m11 = g[3], f0 = g[4], f1 = g[5];
            for (int k = 0; k < 6; ++k)
                sg[k] = g[k];
            const int ozB = min(oz0 + RY_T - 1, nz - 1), oxB = min(ox0 + RY_T - 1, nx - 1);
            double czmin = DBL_MAX, czmax = -DBL_MAX, cxmin = DBL_MAX, cxmax = -DBL_MAX;
            for (int k = 0; k < 4; ++k) {
                const double oz = (k & 1) ? ozB : oz0, oxx = (k & 2) ? oxB : ox0;
                const double cz = (f0 + m00 * oz) + m01 * oxx, cx = (f1 + m10 * oz) + m11 * oxx;
                czmin = fmin(czmin, cz);
                czmax = fmax(czmax, cz);
                cxmin = fmin(cxmin, cx);
                cxmax = fmax(cxmax, cx);
            }
            int zn = 0, xn = 0, z0 = 0, x0 = 0;
            if (!(czmax < -0.01 || czmin > nz - 1 + 0.01 || cxmax < -0.01 || cxmin > nx - 1 + 0.01)) {
                long long zlo = tap_start_d<ORDER>(czmin) - 1, zhi = tap_start_d<ORDER>(czmax) + ORDER + 1;
                long long xlo = tap_start_d<ORDER>(cxmin) - 1, xhi = tap_start_d<ORDER>(cxmax) + ORDER + 1;
                zlo = zlo < 0 ? 0 : zlo;
                xlo = xlo < 0 ? 0 : xlo;
                zhi = zhi > nz - 1 ? nz - 1 : zhi;
                xhi = xhi > nx - 1 ? nx - 1 : xhi;
                z0 = (int)zlo;
                x0 = (int)xlo;
                zn = (int)(zhi - zlo + 1);
                xn = (int)(xhi - xlo + 1);
                if (zn > RY_BOX || xn > RY_BOX) {
                    atomicOr(R.status, DEVCHK_BOX_OVERFLOW);
                    zn = 0;
                }
            }
            const double cz0 = (f0 + m00 * (double)oz0) + m01 * (double)ox0;
            const double cx0 = (f1 + m10 * (double)oz0) + m11 * (double)ox0;
            sax[0] = make_axis(cz0, m00, m01);
            sax[1] = make_axis(cx0, m10, m11);
            si[0] = z0;
            si[1] = x0;
            si[2] = zn;
            si[3] = xn;
        }
        __syncthreads();
        const int zn = si[2];
        if (zn > 0) {
            const int bz0 = si[0], bx0 = si[1], xn = si[3];
            const float2 *plane = slab + ((size_t)a * ny + y) * (size_t)nz * nx;
            for (int zi = ty; zi < zn; zi += 8) {
                const float2 *row = plane + (size_t)(bz0 + zi) * nx + bx0;
                for (int xi = tx; xi < xn; xi += 32)
                    box[zi * RY_BP + xi] = __ldg(row + xi);
            }
            __syncthreads();
            const AxisCoord az = sax[0], ax = sax[1];
            const float dx = (float)(ox - ox0);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int oz = oz0 + ty + 8 * q;
                if (oz >= nz || ox >= nx)
                    continue;
                const float dz = (float)(oz - oz0);
                int Iz, Ix;
                const float lz = eval_axis(az, dz, dx, Iz);
                const float lx = eval_axis(ax, dz, dx, Ix);
                const bool in_z = inside_axis(lz, Iz, nz, [&] {
                    return __dadd_rn(__dadd_rn(sg[4], __dmul_rn(sg[0], (double)oz)), __dmul_rn(sg[1], (double)ox));
                });
                if (!in_z)
                    continue;
                const bool in_x = inside_axis(lx, Ix, nx, [&] {
                    return __dadd_rn(__dadd_rn(sg[5], __dmul_rn(sg[2], (double)oz)), __dmul_rn(sg[3], (double)ox));
                });
                if (!in_x)
                    continue;
                int tz0, tx0;
                float wz[ORDER + 1], wx[ORDER + 1];
                if (ORDER == 0) {
                    // nearest neighbour: the rounding point is a discontinuity,
                    // so take the tap from the exact FP64 coordinate
                    const double cz = __dadd_rn(__dadd_rn(sg[4], __dmul_rn(sg[0], (double)oz)),
                                                __dmul_rn(sg[1], (double)ox));
                    const double cx = __dadd_rn(__dadd_rn(sg[5], __dmul_rn(sg[2], (double)oz)),
                                                __dmul_rn(sg[3], (double)ox));
                    tz0 = (int)floor(cz + 0.5);
                    tx0 = (int)floor(cx + 0.5);
                    wz[0] = 1.f;
                    wx[0] = 1.f;
                } else {
                    tz0 = Iz + Spline<ORDER>::weights(lz, wz);
                    tx0 = Ix + Spline<ORDER>::weights(lx, wx);
                }
                int cx[ORDER + 1];
#pragma unroll
                for (int k = 0; k <= ORDER; ++k)
                    cx[k] = mirror_idx(tx0 + k, nx) - bx0;
                float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                for (int i = 0; i <= ORDER; ++i) {
                    const float2 *brow = box + (mirror_idx(tz0 + i, nz) - bz0) * RY_BP;
                    float2 r = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k <= ORDER; ++k) {
                        const float2 b = brow[cx[k]];
                        r.x = fmaf(wx[k], b.x, r.x);
                        if (!ONLYREAL)
                            r.y = fmaf(wx[k], b.y, r.y);
                    }
                    acc.x = fmaf(wz[i], r.x, acc.x);
                    if (!ONLYREAL)
                        acc.y = fmaf(wz[i], r.y, acc.y);
                }
                kahan_add(s[q], cp[q], acc);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int oz = oz0 + ty + 8 * q;
        if (oz < nz && ox < nx)
            store_sum<ONLYREAL>(R, volume, comp, ((size_t)oz * ny + y) * nx + ox, s[q], cp[q]);
    }
}

// ---------------------------------------------------------------------------
// Tilted path: 3D affine resampling in the reference's (x, -y, z) frame.
// Slab layout [a][z][y][x].  Output voxel (z, y, x) <- frame point
// o = (x, ny-1-y, z); coordinate c = M o + off (scipy order); taps are read
// back through the same mapping.
template <int ORDER, bool ONLYREAL>
__global__ void __launch_bounds__(256) k_rotate_3d(RotParams R, const float2 *__restrict__ slab,
                                                   const double *__restrict__ geo, void *volume, float2 *comp)
{
    __shared__ double sg[12];
    __shared__ AxisCoord sax[3];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8, z = blockIdx.z;
    const int nx = R.nx, ny = R.ny, nz = R.nz;
    const int x = x0 + tx, y = y0 + ty;
    const bool valid = x < nx && y < ny;
    const int n[3] = {nx, ny, nz};
    float2 s = make_float2(0.f, 0.f), cp = make_float2(0.f, 0.f);
    const double o0 = (double)x, o1 = (double)(ny - 1 - y), o2 = (double)z;
    for (int a = 0; a < R.nbatch_angles; ++a) {
        if (threadIdx.x == 0) {
            const double *g = geo + 12 * (size_t)a;
            for (int k = 0; k < 12; ++k)
                sg[k] = g[k];
            const double b0 = (double)x0, b1 = (double)(ny - 1 - y0), b2 = (double)z;
            for (int i = 0; i < 3; ++i) {
                const double c = ((g[9 + i] + g[3 * i] * b0) + g[3 * i + 1] * b1) + g[3 * i + 2] * b2;
                sax[i] = make_axis(c, g[3 * i], g[3 * i + 1]);
            }
        }
        __syncthreads();
        if (valid) {
            const float d0 = (float)tx, d1 = (float)(-ty);
            float l[3];
            int Ib[3];
            bool inside = true;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                l[i] = eval_axis(sax[i], d0, d1, Ib[i]);
                inside = inside && inside_axis(l[i], Ib[i], n[i], [&] {
                    return __dadd_rn(__dadd_rn(__dadd_rn(sg[9 + i], __dmul_rn(sg[3 * i], o0)),
                                               __dmul_rn(sg[3 * i + 1], o1)),
                                     __dmul_rn(sg[3 * i + 2], o2));
                });
            }
            if (inside) {
                int t0[3];
                float w[3][ORDER + 1];
                if (ORDER == 0) {
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const double c = __dadd_rn(__dadd_rn(__dadd_rn(sg[9 + i], __dmul_rn(sg[3 * i], o0)),
                                                             __dmul_rn(sg[3 * i + 1], o1)),
                                                   __dmul_rn(sg[3 * i + 2], o2));
                        t0[i] = (int)floor(c + 0.5);
                        w[i][0] = 1.f;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 3; ++i)
                        t0[i] = Ib[i] + Spline<ORDER>::weights(l[i], w[i]);
                }
                int ix[ORDER + 1], iy[ORDER + 1], iz[ORDER + 1];
#pragma unroll
                for (int k = 0; k <= ORDER; ++k) {
                    ix[k] = mirror_idx(t0[0] + k, nx);
                    iy[k] = ny - 1 - mirror_idx(t0[1] + k, ny);
                    iz[k] = mirror_idx(t0[2] + k, nz);
                }
                const float2 *base = slab + (size_t)a * nz * ny * nx;
                float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                for (int c2 = 0; c2 <= ORDER; ++c2) {
                    float2 r1 = make_float2(0.f, 0.f);
#pragma unroll
                    for (int c1 = 0; c1 <= ORDER; ++c1) {
                        const float2 *row = base + ((size_t)iz[c2] * ny + iy[c1]) * nx;
                        float2 r0 = make_float2(0.f, 0.f);
#pragma unroll
                        for (int c0 = 0; c0 <= ORDER; ++c0) {
                            const float2 b = __ldg(row + ix[c0]);
                            r0.x = fmaf(w[0][c0], b.x, r0.x);
                            r0.y = fmaf(w[0][c0], b.y, r0.y);
                        }
                        r1.x = fmaf(w[1][c1], r0.x, r1.x);
                        r1.y = fmaf(w[1][c1], r0.y, r1.y);
                    }
                    acc.x = fmaf(w[2][c2], r1.x, acc.x);
                    acc.y = fmaf(w[2][c2], r1.y, acc.y);
                }
                kahan_add(s, cp, acc);
            }
        }
        __syncthreads();
    }
    if (valid)
        store_sum<ONLYREAL>(R, volume, comp, ((size_t)z * ny + y) * nx + x, s, cp);
}

template <int ORDER, bool ONLYREAL>
static cudaError_t rotate_impl(const RotParams &R, int tilted, const float2 *slab, const double *geo, void *volume,
                               float2 *comp, cudaStream_t s)
{
    if (!tilted) {
        dim3 grid((R.nx + RY_T - 1) / RY_T, (R.nz + RY_T - 1) / RY_T, R.ny);
        k_rotate_y<ORDER, ONLYREAL><<<grid, 256, 0, s>>>(R, slab, geo, volume, comp);
    } else {
        dim3 grid((R.nx + 31) / 32, (R.ny + 7) / 8, R.nz);
        k_rotate_3d<ORDER, ONLYREAL><<<grid, 256, 0, s>>>(R, slab, geo, volume, comp);
    }
    return cudaGetLastError();
}

cudaError_t launch_rotate(const RotParams &R, int order, int tilted, const float2 *slab, const double *geo,
                          void *volume, float2 *comp, cudaStream_t s)
{
#define ODT_ROT_CASE(O)                                                              \
    case O:                                                                          \
        return R.onlyreal ? rotate_impl<O, true>(R, tilted, slab, geo, volume, comp, s) \
                          : rotate_impl<O, false>(R, tilted, slab, geo, volume, comp, s);
    switch (order) {
        ODT_ROT_CASE(0)
        ODT_ROT_CASE(1)
        ODT_ROT_CASE(2)
        ODT_ROT_CASE(3)
    default:
        return cudaErrorInvalidValue;
    }
#undef ODT_ROT_CASE
}

}  // namespace odt
