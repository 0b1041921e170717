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
#include <limits.h>
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "odt_fft.cuh"
#include "odt_internal.cuh"
#include "odt_tma.cuh"

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

// Quartic and quintic centred B-splines, as polynomials in the fraction t
// (the piecewise forms of the B-spline of degree 4 and 5).
template <>
struct Spline<4> {
    __device__ static int weights(float c, float *w)
    {
        const float s = floorf(c + 0.5f);
        const float t = c - s;  // [-0.5, 0.5)
        const float a = 1.f - 2.f * t, b = 1.f + 2.f * t, a2 = a * a, b2 = b * b, t2 = t * t;
        auto mid = [](float u) {  // 0.5 <= u <= 1.5
            const float u2 = u * u;
            return (55.f + 20.f * u - 120.f * u2 + 80.f * u2 * u - 16.f * u2 * u2) * (1.f / 96.f);
        };
        w[0] = a2 * a2 * (1.f / 384.f);
        w[1] = mid(1.f + t);
        w[2] = 115.f / 192.f - 0.625f * t2 + 0.25f * t2 * t2;
        w[3] = mid(1.f - t);
        w[4] = b2 * b2 * (1.f / 384.f);
        return (int)s - 2;
    }
};
template <>
struct Spline<5> {
    __device__ static int weights(float c, float *w)
    {
        const float s = floorf(c);
        const float t = c - s;  // [0, 1)
        auto inner = [](float d) {  // 0 <= d <= 1
            const float d2 = d * d;
            return 0.55f - 0.5f * d2 + 0.25f * d2 * d2 - d2 * d2 * d * (1.f / 12.f);
        };
        auto mid = [](float d) {  // 1 <= d <= 2
            const float d2 = d * d;
            return 0.425f + 0.625f * d - 1.75f * d2 + 1.25f * d2 * d - 0.375f * d2 * d2 + d2 * d2 * d * (1.f / 24.f);
        };
        const float u = 1.f - t, u2 = u * u, t2 = t * t;
        w[0] = u2 * u2 * u * (1.f / 120.f);
        w[1] = mid(1.f + t);
        w[2] = inner(t);
        w[3] = inner(u);
        w[4] = mid(2.f - t);
        w[5] = t2 * t2 * t * (1.f / 120.f);
        return (int)s - 2;
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
// y-axis path: every (z, x) plane at fixed y is rotated by the same 2D map,
// so the weights and taps of an output (z, x) are the same for all y.  The
// slab layout is [a][z][x][y] (y innermost, pitch R.ypitch); a group of
// lanes shares an output and each lane holds 2 consecutive y, so every tap
// read is one contiguous, conflict-free row of shared memory read as
// 16-byte loads, and the per-output work (coordinates, in/out decision,
// weights) is done once per group.
//
// Work split: a CTA owns a 16 (z) x 16 (x) output tile and Y values of y
// and loops over the batch's angles.  Per angle, the footprint of the
// rotated tile is staged in shared memory -- by one bulk tensor (TMA) copy
// when every footprint position is inside the slab, else by a cp.async
// gather -- double-buffered so that the next angle's footprint streams in
// while the current one is interpolated.  Footprint positions are virtual:
// positions outside [0, n-1] are filled from their mirror images, so the
// interpolation itself never mirrors.  Threads 0..255 compute the parameter
// record (box offset, in/out flag, weights) of one output each per angle.
constexpr int R2_T = 16;        // output tile 16 (z) x 16 (x)
constexpr int R2_THREADS = 512;
constexpr int R2_KAHAN = 8;     // angles summed plainly between Kahan steps
constexpr int R2_RING = 4;      // tile records in flight (angles a..a+3)
constexpr int R2_WMAX = 6;      // spline taps per axis, up to order 5
// Shape of the y-axis resampling per spline order.  A footprint spans the
// tap starts of the tile's outputs (their coordinates span at most
// 15 (|cos| + |sin|) <= 15 sqrt(2), so at most 22 starts), plus the ORDER + 1
// taps and one position of margin on each side: at most 25 + ORDER
// positions per axis (k_rotate_y_setup checks it).  Orders <= 3: 16 y per
// CTA; orders 4 and 5 (30 x 30) take 8 y to keep two footprint buffers in
// shared memory.  LPO lanes (2 y each) share an output.  The parameter
// record of an output: 4 words (box offset, in/out flag), then the z and x
// weights, each duplicated into a (w, w) pair for packed FMAs; at least 20
// words (80 bytes), so that the 16-byte stores of 8 consecutive threads hit
// disjoint banks.  Where two record buffers fit next to the two footprint
// buffers (every order but 3), the records of angle a+1 are computed while
// angle a is interpolated (DBL), with one barrier per angle.
template <int ORDER>
struct RotY {
    static constexpr int Y = ORDER >= 4 ? 8 : 16;              // y values per CTA
    static constexpr int BOX = ORDER >= 4 ? 30 : 25 + ORDER;   // max footprint per axis (virtual positions)
    static constexpr int BOXE = BOX * BOX * Y;                 // float2 per footprint buffer
    static constexpr int LPO = Y / 2;                          // lanes per output
    static constexpr int OUTW = R2_T * R2_T * LPO / R2_THREADS;  // outputs per thread
    static constexpr int SUMS = 2 * OUTW;                      // (output, y) sums per thread
    static constexpr int PW = 4 + 4 * (ORDER + 1) > 20 ? 4 + 4 * (ORDER + 1) : 20;
    static constexpr size_t PRM = (size_t)R2_T * R2_T * PW * sizeof(float);  // one record buffer
    static constexpr size_t FIXED = (size_t)2 * BOXE * sizeof(float2) + (size_t)R2_RING * 64 + 2 * sizeof(uint64_t);
    static constexpr bool DBL = FIXED + 2 * PRM <= 227 * 1024;
    static constexpr size_t SMEM = FIXED + (DBL ? 2 : 1) * PRM;
};

// Footprints whose positions are all inside the slab (no mirrored
// positions) are copied by the TMA unit: one bulk tensor copy per angle of
// a [zb][xb][Y y] box, zb and xb the smallest of three box sizes that hold
// the footprint (the extra positions are real slab positions or zero fill
// and are never read).  The slab of a batch is a 4D tensor map (y, x, z,
// angle) per box shape; boundary footprints keep the cp.async gather, which
// fills mirrored positions from their images.  Measured on the 256^3
// resampling: 15.65 ms with the cp.async gather only, 13.52 ms with TMA.
constexpr bool kRotateTma = true;
constexpr int R2_NTMA = 3;
// TMA box sizes per axis: the footprint bound and two smaller shapes
template <int ORDER>
__host__ __device__ constexpr int r2_tma_box(int i)
{
    return RotY<ORDER>::BOX - 4 * (R2_NTMA - 1 - i);
}
struct RotMaps {
    CUtensorMap m[R2_NTMA * R2_NTMA];  // [z box][x box]
};
// wait for a bulk tensor copy: ~1 s of global time at most
constexpr uint64_t kCopyWaitNs = 1000000000ull;

// d = a * b + c on (re, im) pairs: one packed FP32 FMA
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;\n"
        : "=l"(d)
        : "l"(*reinterpret_cast<unsigned long long *>(&a)), "l"(*reinterpret_cast<unsigned long long *>(&b)),
          "l"(*reinterpret_cast<unsigned long long *>(&c)));
    return *reinterpret_cast<float2 *>(&d);
}

struct __align__(16) TileGeo {
    AxisCoord z, x;            // coordinates at the tile origin
    short box_z0, box_x0;      // footprint origin (virtual: may be < 0)
    short box_zn, box_xn;      // footprint size; box_zn == 0: no output of
                               // the tile is inside for this angle
    short interior;            // every output of the tile inside with margin:
                               // no in/out decisions needed
    short box_real;            // every footprint position in [0, n-1]
    int pad;
};
static_assert(sizeof(TileGeo) == 64, "TileGeo is one 64-byte record");

template <int ORDER, bool TMA>
__global__ void k_rotate_y_setup(RotParams R, const double *__restrict__ geo, TileGeo *__restrict__ tiles)
{
    const int ntz = (R.nz + R2_T - 1) / R2_T, ntx = (R.nx + R2_T - 1) / R2_T;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= R.nbatch_angles * ntz * ntx)
        return;
    const int a = id / (ntz * ntx), t = id % (ntz * ntx);
    const int oz0 = (t / ntx) * R2_T, ox0 = (t % ntx) * R2_T;
    const int nz = R.nz, nx = R.nx;
    const double *g = geo + 6 * (size_t)a;
    const double m00 = g[0], m01 = g[1], m10 = g[2], m11 = g[3], f0 = g[4], f1 = g[5];
    const int ozB = min(oz0 + R2_T - 1, nz - 1), oxB = min(ox0 + R2_T - 1, nx - 1);
    double czmin = DBL_MAX, czmax = -DBL_MAX, cxmin = DBL_MAX, cxmax = -DBL_MAX;
    for (int k = 0; k < 4; ++k) {
        const double oz = (k & 1) ? ozB : oz0, oxx = (k & 2) ? oxB : ox0;
        const double cz = (f0 + m00 * oz) + m01 * oxx, cx = (f1 + m10 * oz) + m11 * oxx;
        czmin = fmin(czmin, cz);
        czmax = fmax(czmax, cz);
        cxmin = fmin(cxmin, cx);
        cxmax = fmax(cxmax, cx);
    }
    TileGeo tg;
    tg.z = make_axis((f0 + m00 * (double)oz0) + m01 * (double)ox0, m00, m01);
    tg.x = make_axis((f1 + m10 * (double)oz0) + m11 * (double)ox0, m10, m11);
    tg.box_z0 = tg.box_x0 = tg.box_zn = tg.box_xn = 0;
    tg.interior = 0;
    tg.box_real = 0;
    tg.pad = 0;
    // only outputs with coordinates in [0, n-1] are interpolated: their taps
    // span the clamped coordinate range plus the spline support (and one
    // position of margin on each side for FP32 rounding of the tap start)
    const double zlo_c = fmax(czmin, 0.0), zhi_c = fmin(czmax, (double)(nz - 1));
    const double xlo_c = fmax(cxmin, 0.0), xhi_c = fmin(cxmax, (double)(nx - 1));
    if (zlo_c <= zhi_c + 0.01 && xlo_c <= xhi_c + 0.01) {
        const long long zlo = tap_start_d<ORDER>(zlo_c) - 1, zhi = tap_start_d<ORDER>(zhi_c) + ORDER + 1;
        const long long xlo = tap_start_d<ORDER>(xlo_c) - 1, xhi = tap_start_d<ORDER>(xhi_c) + ORDER + 1;
        const long long zn = zhi - zlo + 1, xn = xhi - xlo + 1;
        if (zn > RotY<ORDER>::BOX || xn > RotY<ORDER>::BOX) {
            atomicOr(R.status, DEVCHK_BOX_OVERFLOW);
        } else {
            tg.box_z0 = (short)zlo;
            tg.box_x0 = (short)xlo;
            tg.box_zn = (short)zn;
            tg.box_xn = (short)xn;
            tg.interior = (czmin > 0.01 && czmax < nz - 1 - 0.01 && cxmin > 0.01 && cxmax < nx - 1 - 0.01 &&
                           ozB == oz0 + R2_T - 1 && oxB == ox0 + R2_T - 1)
                              ? 1
                              : 0;
            tg.box_real = (zlo >= 0 && zhi <= nz - 1 && xlo >= 0 && xhi <= nx - 1) ? 1 : 0;
            if (TMA && tg.box_real) {
                // box shape of the TMA copy: rows of the staged box are
                // xb positions apart, so the box size becomes the staged
                // size (tap positions stay inside the true footprint)
                int iz = 0, ix = 0;
                while (r2_tma_box<ORDER>(iz) < zn)
                    ++iz;
                while (r2_tma_box<ORDER>(ix) < xn)
                    ++ix;
                tg.box_zn = (short)r2_tma_box<ORDER>(iz);
                tg.box_xn = (short)r2_tma_box<ORDER>(ix);
                tg.pad = 1 + iz * R2_NTMA + ix;
            }
        }
    }
    tiles[id] = tg;
}


// Issue the footprint copy of one (angle, tile) for y values [y0, y0+Y):
// position p = (vz, vx) of the box holds Y y at buf[p*Y .. p*Y+Y-1], read
// from the mirror image of (vz, vx).  Thread t copies 16-byte part t % (Y/2)
// of positions t / (Y/2) + k * (threads / (Y/2)).
template <int Y>
__device__ __forceinline__ void stage_box(const TileGeo &tg, const float2 *aslab, int nz, int nx, int ypitch,
                                          int y0, float2 *buf)
{
    constexpr int PARTS = Y / 2, R2_Y = Y;
    const int zn = tg.box_zn, xn = tg.box_xn, np = zn * xn;
    const int part = threadIdx.x % PARTS;
    int pidx = threadIdx.x / PARTS;
    if (pidx >= np)
        return;
    constexpr int step = R2_THREADS / PARTS;  // positions per pass
    const int sq = step / xn, sr = step % xn;
    int pz = pidx / xn, px = pidx % xn;
    if (tg.box_real) {
        // every position is real: walk the source address incrementally
        const float2 *src = aslab + ((size_t)(tg.box_z0 + pz) * nx + tg.box_x0 + px) * ypitch + y0 + 2 * part;
        const long long dstep = ((long long)sq * nx + sr) * ypitch, dwrap = (long long)(nx - xn) * ypitch;
        float2 *dst = buf + pidx * R2_Y + 2 * part;
        for (; pidx < np; pidx += step) {
            cp_async16(dst, src);
            dst += step * R2_Y;
            src += dstep;
            px += sr;
            if (px >= xn) {
                px -= xn;
                src += dwrap;
            }
        }
        return;
    }
    for (; pidx < np; pidx += step) {
        const int mz = mirror_idx(tg.box_z0 + pz, nz), mx = mirror_idx(tg.box_x0 + px, nx);
        cp_async16(buf + pidx * R2_Y + 2 * part, aslab + ((size_t)mz * nx + mx) * ypitch + y0 + 2 * part);
        px += sr;
        pz += sq;
        if (px >= xn) {
            px -= xn;
            ++pz;
        }
    }
}

__device__ __forceinline__ TileGeo load_tile(const TileGeo *p)
{
    TileGeo t;
    const int4 *s = reinterpret_cast<const int4 *>(p);
    int4 *d = reinterpret_cast<int4 *>(&t);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        d[k] = s[k];
    return t;
}

// Taps of output (oz, ox) for one angle: the position (rz, rx) of its first
// tap in the tile's footprint box and the z and x weights.  False (weights
// zero) for an output outside the domain, or whose taps leave the box (then
// recorded in the status word).
template <int ORDER>
__device__ __forceinline__ bool output_taps(const RotParams &R, const TileGeo &cur, const double *g, int oz0,
                                            int ox0, int oz, int ox, int &rz, int &rx, float (&wz)[R2_WMAX],
                                            float (&wx)[R2_WMAX])
{
    bool ok = false;
    rz = rx = 0;
#pragma unroll
    for (int k = 0; k < R2_WMAX; ++k)
        wz[k] = wx[k] = 0.f;
    const int nz = R.nz, nx = R.nx;
    if (cur.box_zn > 0 && oz < nz && ox < nx) {
        int Iz, Ix;
        const float dz = (float)(oz - oz0), dx = (float)(ox - ox0);
        const float lz = eval_axis(cur.z, dz, dx, Iz);
        const float lx = eval_axis(cur.x, dz, dx, Ix);
        bool in = true;
        if (!cur.interior) {
            in = inside_axis(lz, Iz, nz, [&] {
                return __dadd_rn(__dadd_rn(__ldg(g + 4), __dmul_rn(__ldg(g + 0), (double)oz)),
                                 __dmul_rn(__ldg(g + 1), (double)ox));
            });
            in = in && inside_axis(lx, Ix, nx, [&] {
                return __dadd_rn(__dadd_rn(__ldg(g + 5), __dmul_rn(__ldg(g + 2), (double)oz)),
                                 __dmul_rn(__ldg(g + 3), (double)ox));
            });
        }
        if (in) {
            int tz0, tx0;
            if (ORDER == 0) {
                // nearest neighbour: the rounding point is a discontinuity,
                // so take the tap from the exact FP64 coordinate
                const double cz = __dadd_rn(__dadd_rn(__ldg(g + 4), __dmul_rn(__ldg(g + 0), (double)oz)),
                                            __dmul_rn(__ldg(g + 1), (double)ox));
                const double cx = __dadd_rn(__dadd_rn(__ldg(g + 5), __dmul_rn(__ldg(g + 2), (double)oz)),
                                            __dmul_rn(__ldg(g + 3), (double)ox));
                tz0 = (int)floor(cz + 0.5);
                tx0 = (int)floor(cx + 0.5);
                wz[0] = 1.f;
                wx[0] = 1.f;
            } else {
                float w[ORDER + 1];
                tz0 = Iz + Spline<ORDER>::weights(lz, w);
#pragma unroll
                for (int k = 0; k <= ORDER; ++k)
                    wz[k] = w[k];
                tx0 = Ix + Spline<ORDER>::weights(lx, w);
#pragma unroll
                for (int k = 0; k <= ORDER; ++k)
                    wx[k] = w[k];
            }
            rz = tz0 - cur.box_z0;
            rx = tx0 - cur.box_x0;
            if (rz >= 0 && rz + ORDER < cur.box_zn && rx >= 0 && rx + ORDER < cur.box_xn) {
                ok = true;
            } else {
                atomicOr(R.status, DEVCHK_BOX_OVERFLOW);  // tap outside the staged box
#pragma unroll
                for (int k = 0; k < R2_WMAX; ++k)
                    wz[k] = wx[k] = 0.f;
            }
        }
    }
    return ok;
}

// Parameter record of output (oz, ox) for one angle: word 0 box offset of
// the first tap (float2 units), word 1 in/out flag, then (wz_i, wz_i) pairs
// and (wx_k, wx_k) pairs, i, k = 0..ORDER.
template <int ORDER>
__device__ __forceinline__ void output_params(const RotParams &R, const TileGeo &cur, const double *g, int oz0,
                                              int ox0, int oz, int ox, float *rec)
{
    int rz, rx;
    float wz[R2_WMAX], wx[R2_WMAX];
    const int ok = output_taps<ORDER>(R, cur, g, oz0, ox0, oz, ox, rz, rx, wz, wx) ? 1 : 0;
    const int off = ok ? (rz * cur.box_xn + rx) * RotY<ORDER>::Y : 0;
    // 16-byte stores only: header, then the (w, w) pairs two per store
    float w[2 * (ORDER + 1) + 1];
#pragma unroll
    for (int k = 0; k <= ORDER; ++k) {
        w[k] = wz[k];
        w[ORDER + 1 + k] = wx[k];
    }
    w[2 * (ORDER + 1)] = 0.f;
    float4 *r4 = reinterpret_cast<float4 *>(rec);
    r4[0] = make_float4(__int_as_float(off), __int_as_float(ok), 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < ORDER + 1; ++k)
        r4[1 + k] = make_float4(w[2 * k], w[2 * k], w[2 * k + 1], w[2 * k + 1]);
}

template <int ORDER, bool ONLYREAL, bool TMA>
__global__ void __launch_bounds__(R2_THREADS, 1) k_rotate_y(RotParams R, const float2 *__restrict__ slab,
                                                            const double *__restrict__ geo,
                                                            const TileGeo *__restrict__ tiles, void *volume,
                                                            float2 *comp, const __grid_constant__ RotMaps maps)
{
    using C = RotY<ORDER>;
    constexpr int R2_Y = C::Y, R2_BOXE = C::BOXE, PW = C::PW, R2_OUT = C::SUMS, LPO = C::LPO;
    extern __shared__ __align__(1024) float4 r2_smem[];
    float2 *box = reinterpret_cast<float2 *>(r2_smem);       // [2][R2_BOXE]
    float *prm = reinterpret_cast<float *>(box + 2 * R2_BOXE); // [DBL ? 2 : 1][256][PW]
    constexpr int PRMN = R2_T * R2_T * PW;  // floats per record buffer
    TileGeo *ring = reinterpret_cast<TileGeo *>(prm + (C::DBL ? 2 : 1) * PRMN);  // [R2_RING]
    uint64_t *bar = reinterpret_cast<uint64_t *>(ring + R2_RING);  // [2]: TMA copies into box[0], box[1]
    unsigned phase = 0;  // bit b: parity of the next TMA completion of box[b]
    const int tid = threadIdx.x;
    // LPO lanes per output (8 for orders <= 3), each with 2 consecutive y:
    // a tap read is one 16-byte load per lane (a 128-byte row per 8 lanes),
    // so a warp reads the taps of 4 outputs per instruction and a record
    // serves 8 lanes (measured on the 256^3 resampling: 13.27 ms with 16
    // lanes of one y per output, 12.04 ms like this)
    constexpr int OUTW = C::OUTW;  // outputs per thread, 2 y each
    const int hw = tid / LPO, yl = (tid % LPO) * 2;
    const int ntx = (R.nx + R2_T - 1) / R2_T, ntz = (R.nz + R2_T - 1) / R2_T;
    const int tile = blockIdx.y * ntx + blockIdx.x;
    const int ox0 = blockIdx.x * R2_T, oz0 = blockIdx.y * R2_T, y0 = blockIdx.z * R2_Y;
    const int nx = R.nx, nz = R.nz, ny = R.ny, yp = R.ypitch;
    const int nb = R.nbatch_angles;
    const size_t aslab_stride = (size_t)nz * nx * yp;
    // this thread's outputs: x = ox0 + (hw & 15), z = oz0 + (hw >> 4) * OUTW + i
    const int hx = hw & 15, hz0 = (hw >> 4) * OUTW;
    float2 s[R2_OUT], cp[R2_OUT], part[R2_OUT];  // [output q][y pair]: 2q, 2q+1
#pragma unroll
    for (int q = 0; q < R2_OUT; ++q) {
        s[q] = make_float2(0.f, 0.f);
        cp[q] = make_float2(0.f, 0.f);
        part[q] = make_float2(0.f, 0.f);
    }
    // tile records: angles 0..2 now; angle a+3 travels with the footprint
    // copy of angle a+1, so a record is in shared memory two angles before
    // its footprint copy is issued
    const size_t rec_stride = (size_t)ntz * ntx;
    if (tid < 12 && tid / 4 < nb)
        reinterpret_cast<int4 *>(ring + tid / 4)[tid % 4] =
            __ldg(reinterpret_cast<const int4 *>(tiles + (size_t)(tid / 4) * rec_stride + tile) + tid % 4);
    if (TMA && tid == 0) {
        mbar_init(bar + 0, 1);
        mbar_init(bar + 1, 1);
        fence_mbar_init();
    }
    __syncthreads();
    // footprint copy of angle aa (record t) into box[b]: one bulk tensor copy
    // issued by thread 0, or the cp.async gather
    auto stage = [&](const TileGeo &t, int aa, int b) {
        if (TMA && t.pad > 0) {
            if (tid == 0) {
                const int mi = t.pad - 1;
                const unsigned bytes = (unsigned)t.box_zn * t.box_xn * R2_Y * sizeof(float2);
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(bar + b, bytes);
                tma_load_4d(box + b * R2_BOXE, &maps.m[mi], bar + b, y0, t.box_x0, t.box_z0, aa);
            }
        } else if (t.box_zn > 0) {
            stage_box<R2_Y>(t, slab + (size_t)aa * aslab_stride, nz, nx, yp, y0, box + b * R2_BOXE);
        }
    };
    // every thread waits for the TMA copy of footprint a; a copy that does
    // not complete within the limit is reported and ends the CTA (all
    // threads together, after a second bounded wait by thread 0 so that no
    // copy is left writing into shared memory).  The vote is the barrier
    // that orders angle a's footprint and records before their use.
    auto footprint_barrier = [&](int a, bool tma_copy) -> bool {
        if (TMA && tma_copy) {
            const bool done = mbar_wait(bar + (a & 1), (phase >> (a & 1)) & 1u, kCopyWaitNs);
            phase ^= 1u << (a & 1);
            if (__syncthreads_or(!done)) {
                if (tid == 0) {
                    atomicOr(R.status, DEVCHK_COPY_TIMEOUT);
                    mbar_wait(bar + (a & 1), ((phase >> (a & 1)) & 1u) ^ 1u, kCopyWaitNs);
                }
                __syncthreads();
                return false;
            }
        } else {
            __syncthreads();
        }
        return true;
    };
    auto prefetch_record = [&](int a) {  // tile record of angle a into the ring
        if (a < nb && tid < 4)
            cp_async16(reinterpret_cast<int4 *>(ring + a % R2_RING) + tid,
                       reinterpret_cast<const int4 *>(tiles + (size_t)a * rec_stride + tile) + tid);
    };
    TileGeo cur = load_tile(ring);
    stage(cur, 0, 0);
    cp_async_commit();
    if constexpr (C::DBL) {
        if (tid < R2_T * R2_T)
            output_params<ORDER>(R, cur, geo, oz0, ox0, oz0 + (tid >> 4), ox0 + (tid & 15), prm + tid * PW);
    }
    for (int a = 0; a < nb; ++a) {
        const float *prm_a = prm + ((C::DBL && (a & 1)) ? PRMN : 0);
        if constexpr (C::DBL) {
            // one barrier per angle: footprint a (copied during angle a-1)
            // and its records (computed during angle a-1) are complete, and
            // every thread is done with angle a-1's footprint and record
            // buffers, which angle a+1 takes now; threads 0..255 compute the
            // records of angle a+1 while the others start interpolating
            cp_async_wait<0>();
            if (!footprint_barrier(a, cur.pad > 0))
                return;
            if (a + 1 < nb) {
                const TileGeo nxt = load_tile(ring + (a + 1) % R2_RING);
                stage(nxt, a + 1, (a + 1) & 1);
                prefetch_record(a + 3);
                cp_async_commit();
                if (tid < R2_T * R2_T)
                    output_params<ORDER>(R, nxt, geo + 6 * (size_t)(a + 1), oz0, ox0, oz0 + (tid >> 4),
                                         ox0 + (tid & 15), prm + ((a + 1) & 1) * PRMN + tid * PW);
            }
        } else {
            if (a + 1 < nb)
                stage(load_tile(ring + (a + 1) % R2_RING), a + 1, (a + 1) & 1);
            prefetch_record(a + 3);
            cp_async_commit();
            if (tid < R2_T * R2_T)
                output_params<ORDER>(R, cur, geo + 6 * (size_t)a, oz0, ox0, oz0 + (tid >> 4), ox0 + (tid & 15),
                                     prm + tid * PW);
            cp_async_wait<1>();
            if (!footprint_barrier(a, cur.pad > 0))
                return;
        }
        if (cur.box_zn > 0) {
            const float2 *b = box + (a & 1) * R2_BOXE + yl;
            const int rowstride = cur.box_xn * R2_Y;
#pragma unroll
            for (int q = 0; q < OUTW; ++q) {
                // no branch on the in/out flag: an output outside the domain
                // has zero weights and box offset 0 (a staged position), so
                // it adds zero, and the loop over q stays straight-line code
                // whose loads the compiler can issue ahead (measured: 13.52
                // -> 13.28 ms for the 256^3 resampling)
                const float *rec = prm_a + ((hz0 + q) * R2_T + hx) * PW;
                const float4 h = *reinterpret_cast<const float4 *>(rec);
                float2 w[2 * (ORDER + 1)];
#pragma unroll
                for (int k = 0; k < 2 * (ORDER + 1); k += 2) {
                    const float4 t4 = *reinterpret_cast<const float4 *>(rec + 4 + 2 * k);
                    w[k] = make_float2(t4.x, t4.y);
                    w[k + 1] = make_float2(t4.z, t4.w);
                }
                const float2 *t = b + __float_as_int(h.x);
                float2 acc0 = part[2 * q], acc1 = part[2 * q + 1];
#pragma unroll
                for (int i = 0; i <= ORDER; ++i) {
                    const float2 *row = t + i * rowstride;
                    float2 r0 = make_float2(0.f, 0.f), r1 = r0;
#pragma unroll
                    for (int k = 0; k <= ORDER; ++k) {
                        const float4 t4 = *reinterpret_cast<const float4 *>(row + k * R2_Y);
                        r0 = ffma2(w[ORDER + 1 + k], make_float2(t4.x, t4.y), r0);
                        r1 = ffma2(w[ORDER + 1 + k], make_float2(t4.z, t4.w), r1);
                    }
                    acc0 = ffma2(w[i], r0, acc0);
                    acc1 = ffma2(w[i], r1, acc1);
                }
                part[2 * q] = acc0;
                part[2 * q + 1] = acc1;
            }
        }
        if ((a % R2_KAHAN) == R2_KAHAN - 1 || a == nb - 1) {
#pragma unroll
            for (int q = 0; q < R2_OUT; ++q) {
                kahan_add(s[q], cp[q], part[q]);
                part[q] = make_float2(0.f, 0.f);
            }
        }
        if constexpr (!C::DBL)
            __syncthreads();  // footprint and record buffers free for angle a+2 / a+1
        if (a + 1 < nb)
            cur = load_tile(ring + (a + 1) % R2_RING);
    }
    const int ox = ox0 + hx;
    if (ox < nx) {
#pragma unroll
        for (int q = 0; q < R2_OUT; ++q) {
            const int oz = oz0 + hz0 + q / 2, y = y0 + yl + (q & 1);
            if (oz < nz && y < ny)
                store_sum<ONLYREAL>(R, volume, comp, ((size_t)oz * ny + y) * nx + ox, s[q], cp[q]);
        }
    }
}

// ---------------------------------------------------------------------------
// Single-row path (ny == 1, the 2D reconstruction): the slab is [a][z][x]
// (pitch 1) and there is no y to spread over lanes, so each of a CTA's 256
// threads owns one output of a 16 x 16 tile and computes its own taps and
// weights (output_taps: the decisions of k_rotate_y).  Per angle the tile's
// footprint (<= 28 x 28 positions, mirrored positions filled from their
// images) is staged in shared memory with 8-byte cp.async, three buffers
// deep: the copies of angles a+1 and a+2 are in flight while angle a is
// interpolated.  The footprint boxes (the last 16 bytes of a tile record)
// are loaded two angles ahead, the whole records one angle ahead.
constexpr int RP_BUFS = 3;

struct BoxDesc {
    short z0, x0, zn, xn, interior, real;
    int pad;
};
static_assert(sizeof(BoxDesc) == 16, "BoxDesc is the 16-byte tail of a TileGeo");

__device__ __forceinline__ BoxDesc load_box(const TileGeo *p)
{
    const int4 v = reinterpret_cast<const int4 *>(p)[3];
    return *reinterpret_cast<const BoxDesc *>(&v);
}

// Issue the footprint copy of one (angle, tile): position (vz, vx) of the
// box at buf[vz * xn + vx], read from its mirror image.
__device__ __forceinline__ void stage_plane(const BoxDesc &b, const float2 *aslab, int nz, int nx, float2 *buf)
{
    const int xn = b.xn, np = b.zn * xn;
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
        const int pz = p / xn, px = p - pz * xn;
        const int mz = b.real ? b.z0 + pz : mirror_idx(b.z0 + pz, nz);
        const int mx = b.real ? b.x0 + px : mirror_idx(b.x0 + px, nx);
        cp_async8(buf + p, aslab + (size_t)mz * nx + mx);
    }
}

template <int ORDER, bool ONLYREAL>
__global__ void __launch_bounds__(R2_T * R2_T) k_rotate_plane(RotParams R, const float2 *__restrict__ slab,
                                                              const double *__restrict__ geo,
                                                              const TileGeo *__restrict__ tiles, void *volume,
                                                              float2 *comp)
{
    constexpr int RP_BOXE = RotY<ORDER>::BOX * RotY<ORDER>::BOX;
    __shared__ float2 box[RP_BUFS][RP_BOXE];
    const int tid = threadIdx.x;
    const int ntx = (R.nx + R2_T - 1) / R2_T, ntz = (R.nz + R2_T - 1) / R2_T;
    const int tile = blockIdx.y * ntx + blockIdx.x;
    const int ox0 = blockIdx.x * R2_T, oz0 = blockIdx.y * R2_T;
    const int ox = ox0 + (tid & (R2_T - 1)), oz = oz0 + tid / R2_T;
    const int nx = R.nx, nz = R.nz, nb = R.nbatch_angles;
    const size_t astride = (size_t)nz * nx, rstride = (size_t)ntz * ntx;
    const TileGeo *trec = tiles + tile;
    float2 s = make_float2(0.f, 0.f), c = s, part = s;
    // angles 0 and 1 staged; records: cur = 0, nxt = 1; box d2 = angle 2
    TileGeo cur = load_tile(trec);
    TileGeo nxt = cur;
    BoxDesc d2 = load_box(trec);
    {
        const BoxDesc b0 = load_box(trec);
        if (b0.zn > 0)
            stage_plane(b0, slab, nz, nx, box[0]);
        cp_async_commit();
        if (nb > 1) {
            nxt = load_tile(trec + rstride);
            const BoxDesc b1 = load_box(trec + rstride);
            if (b1.zn > 0)
                stage_plane(b1, slab + astride, nz, nx, box[1]);
        }
        cp_async_commit();
        if (nb > 2)
            d2 = load_box(trec + 2 * rstride);
    }
    for (int a = 0; a < nb; ++a) {
        TileGeo nxt2 = nxt;
        BoxDesc d3 = d2;
        if (a + 2 < nb) {
            if (d2.zn > 0)
                stage_plane(d2, slab + (size_t)(a + 2) * astride, nz, nx, box[(a + 2) % RP_BUFS]);
            nxt2 = load_tile(trec + (size_t)(a + 2) * rstride);
            if (a + 3 < nb)
                d3 = load_box(trec + (size_t)(a + 3) * rstride);
        }
        cp_async_commit();
        int rz, rx;
        float wz[R2_WMAX], wx[R2_WMAX];
        const bool ok = output_taps<ORDER>(R, cur, geo + 6 * (size_t)a, oz0, ox0, oz, ox, rz, rx, wz, wx);
        cp_async_wait<2>();  // angle a's copies (all but the two latest groups)
        __syncthreads();
        if (ok) {
            const int xn = cur.box_xn;
            const float2 *t = box[a % RP_BUFS] + rz * xn + rx;
            float2 acc = part;
#pragma unroll
            for (int i = 0; i <= ORDER; ++i) {
                float2 r = make_float2(0.f, 0.f);
#pragma unroll
                for (int k = 0; k <= ORDER; ++k)
                    r = ffma2(make_float2(wx[k], wx[k]), t[i * xn + k], r);
                acc = ffma2(make_float2(wz[i], wz[i]), r, acc);
            }
            part = acc;
        }
        if ((a % R2_KAHAN) == R2_KAHAN - 1 || a == nb - 1) {
            kahan_add(s, c, part);
            part = make_float2(0.f, 0.f);
        }
        __syncthreads();  // box[a % 3] is refilled with angle a + 3 next
        cur = nxt;
        nxt = nxt2;
        d2 = d3;
    }
    if (oz < nz && ox < nx)
        store_sum<ONLYREAL>(R, volume, comp, (size_t)oz * nx + ox, s, c);
}

// ---------------------------------------------------------------------------
// Tilted path: 3D affine resampling in the reference's (x, -y, z) frame.
// Output voxel (z, y, x) <- frame point o = (x, ny-1-y, z); coordinate
// c = M o + off (scipy order); tap (t0, t1, t2) is read back through the
// same mapping: slab[a][mirror(t2)][mirror(t0)][ny-1-mirror(t1)] in the
// layout [a][z][x][y] (y innermost, pitch R.ypitch).
//
// Work split: a CTA owns 32 y (the lanes) x 8 x (the warps) x 2 z (per
// thread) outputs.  The rotation axis is close to y, so the frame point of
// consecutive y moves almost along the slab's y axis: the 32 lanes of a tap
// load read one nearly contiguous 256-byte run, served by L1 for the
// neighbouring outputs that share it.  Per angle, the FP32 coordinate
// splits of the tile origin (three axes) and an "interior" flag (every tap
// of every output in range: no in/out decisions, no mirroring) are computed
// once per CTA in FP64 and kept in shared memory for a chunk of angles; the
// splits are read from there at each use (broadcast loads) rather than held
// in registers, which keeps the kernel at 64 registers and 4 CTAs per SM:
// the tap loads are latency bound, and the extra warps hide more of it.
constexpr int R3_Y = 32, R3_X = 8, R3_Z = 2;
// interior margins of the coordinate range: [R3_LO, n - R3_HI]
template <int ORDER>
constexpr double R3_LO = ORDER >= 4 ? 3.0 : 2.0;
template <int ORDER>
constexpr double R3_HI = ORDER >= 5 ? 5.0 : (ORDER >= 4 ? 4.0 : 3.0);
constexpr int R3_CHUNK = 64;
constexpr int R3_KAHAN = 8;

// c(d) = I + f + sum_j m_j d_j for small integer offsets d (three slopes,
// split as in AxisCoord).
struct AxisCoord3 {
    float f, mh0, ml0, mh1, ml1, mh2, ml2;
    int I;
};

__device__ __forceinline__ AxisCoord3 make_axis3(double c0, double m0, double m1, double m2)
{
    AxisCoord3 a;
    const double I = floor(c0);
    a.I = (int)I;
    a.f = (float)(c0 - I);
    const double h0 = rint(m0 * 4096.0) / 4096.0, h1 = rint(m1 * 4096.0) / 4096.0, h2 = rint(m2 * 4096.0) / 4096.0;
    a.mh0 = (float)h0;
    a.ml0 = (float)(m0 - h0);
    a.mh1 = (float)h1;
    a.ml1 = (float)(m1 - h1);
    a.mh2 = (float)h2;
    a.ml2 = (float)(m2 - h2);
    return a;
}

__device__ __forceinline__ float eval_axis3(const AxisCoord3 &a, float d0, float d1, float d2, int &B)
{
    const float S = fmaf(a.mh2, d2, fmaf(a.mh1, d1, a.mh0 * d0));  // exact
    const float Rr = fmaf(a.ml2, d2, fmaf(a.ml1, d1, fmaf(a.ml0, d0, a.f)));
    const float Sf = floorf(S);
    B = a.I + (int)Sf;
    return (S - Sf) + Rr;
}

template <int ORDER, bool ONLYREAL>
__global__ void __launch_bounds__(256, ORDER >= 4 ? 2 : 4) k_rotate_3d(RotParams R, const float2 *__restrict__ slab,
                                                   const double *__restrict__ geo, void *volume, float2 *comp)
{
    __shared__ AxisCoord3 srec[R3_CHUNK][3];
    __shared__ int sflag[R3_CHUNK][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nx = R.nx, ny = R.ny, nz = R.nz, yp = R.ypitch;
    const int x0 = blockIdx.x * R3_X, y0 = blockIdx.y * R3_Y, z0 = blockIdx.z * R3_Z;
    const int x = x0 + w, y = y0 + lane;
    const bool vxy = x < nx && y < ny;
    const bool full = x0 + R3_X <= nx && y0 + R3_Y <= ny && z0 + R3_Z <= nz;
    const int n3[3] = {nx, ny, nz};
    const size_t aslab = (size_t)nz * nx * yp;
    // element offsets within one angle's slab fit 32 bits (plan creation
    // refuses slabs of 2^31 or more elements), so the tap addresses are
    // 32-bit offsets from the angle's slab pointer
    const int zstride = nx * yp;
    // frame offsets of this thread's outputs from the tile origin
    const float d0 = (float)w, d1 = (float)(-lane);
    const double o0 = (double)x, o1 = (double)(ny - 1 - y);
    float2 s[R3_Z], cp[R3_Z], part[R3_Z];
#pragma unroll
    for (int q = 0; q < R3_Z; ++q) {
        s[q] = make_float2(0.f, 0.f);
        cp[q] = make_float2(0.f, 0.f);
        part[q] = make_float2(0.f, 0.f);
    }
    const int nb = R.nbatch_angles;
    for (int a0 = 0; a0 < nb; a0 += R3_CHUNK) {
        const int na = min(R3_CHUNK, nb - a0);
        __syncthreads();
        for (int t = threadIdx.x; t < na * 3; t += blockDim.x) {
            const int aa = t / 3, i = t % 3;
            const double *g = geo + 12 * (size_t)(a0 + aa);
            const double m0 = g[3 * i], m1 = g[3 * i + 1], m2 = g[3 * i + 2];
            const double c = ((g[9 + i] + m0 * (double)x0) + m1 * (double)(ny - 1 - y0)) + m2 * (double)z0;
            srec[aa][i] = make_axis3(c, m0, m1, m2);
            // coordinate range over the tile: o - o_origin in
            // [0, X-1] x [-(Y-1), 0] x [0, Z-1]
            const double e0 = m0 * (R3_X - 1), e1 = -m1 * (R3_Y - 1), e2 = m2 * (R3_Z - 1);
            const double lo = c + fmin(e0, 0.0) + fmin(e1, 0.0) + fmin(e2, 0.0);
            const double hi = c + fmax(e0, 0.0) + fmax(e1, 0.0) + fmax(e2, 0.0);
            // every tap of every output in range (taps from floor(c + 1/2)
            // - ORDER/2 or floor(c) - ORDER/2, ORDER + 1 of them), with one
            // position of margin
            sflag[aa][i] = (full && lo >= R3_LO<ORDER> && hi <= n3[i] - R3_HI<ORDER>) ? 1 : 0;
        }
        __syncthreads();
        for (int aa = 0; aa < na; ++aa) {
            const int a = a0 + aa;
            const bool interior = sflag[aa][0] && sflag[aa][1] && sflag[aa][2];
            const AxisCoord3 *axp = srec[aa];
            const float2 *sa = slab + (size_t)a * aslab;
            const double *g = geo + 12 * (size_t)a;
#pragma unroll
            for (int q = 0; q < R3_Z; ++q) {
                const int z = z0 + q;
                if (!vxy || z >= nz)
                    continue;
                const float d2 = (float)q;
                int Ib[3];
                float l[3];
                l[0] = eval_axis3(axp[0], d0, d1, d2, Ib[0]);
                l[1] = eval_axis3(axp[1], d0, d1, d2, Ib[1]);
                l[2] = eval_axis3(axp[2], d0, d1, d2, Ib[2]);
                const double o2 = (double)z;
                auto exact = [&](int i) {
                    return __dadd_rn(__dadd_rn(__dadd_rn(__ldg(g + 9 + i), __dmul_rn(__ldg(g + 3 * i), o0)),
                                               __dmul_rn(__ldg(g + 3 * i + 1), o1)),
                                     __dmul_rn(__ldg(g + 3 * i + 2), o2));
                };
                if (!interior) {
                    bool in = true;
#pragma unroll
                    for (int i = 0; i < 3; ++i)
                        in = in && inside_axis(l[i], Ib[i], n3[i], [&] { return exact(i); });
                    if (!in)
                        continue;
                }
                int t0[3];
                float wt[3][ORDER + 1];
                if (ORDER == 0) {
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        t0[i] = (int)floor(exact(i) + 0.5);
                        wt[i][0] = 1.f;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 3; ++i)
                        t0[i] = Ib[i] + Spline<ORDER>::weights(l[i], wt[i]);
                }
                float2 acc = part[q];
                // every tap of this output inside the slab (all of them in an
                // interior tile; elsewhere most outputs away from the slab's
                // faces): plain addressing, the same loads in the same order
                // as the mirrored path below
                bool direct = interior;
                if (!interior) {
                    direct = true;
#pragma unroll
                    for (int i = 0; i < 3; ++i)
                        direct = direct && t0[i] >= 0 && t0[i] + ORDER <= n3[i] - 1;
                }
                if (direct) {
                    const int off = (t0[2] * nx + t0[0]) * yp + (ny - 1 - t0[1]);
#pragma unroll
                    for (int k2 = 0; k2 <= ORDER; ++k2) {
#pragma unroll
                        for (int k0 = 0; k0 <= ORDER; ++k0) {
                            const float2 *col = sa + (off + k2 * zstride + k0 * yp);
                            float2 r = make_float2(0.f, 0.f);
#pragma unroll
                            for (int k1 = 0; k1 <= ORDER; ++k1)
                                r = ffma2(make_float2(wt[1][k1], wt[1][k1]), __ldg(col - k1), r);
                            const float w02 = wt[2][k2] * wt[0][k0];
                            acc = ffma2(make_float2(w02, w02), r, acc);
                        }
                    }
                } else {
                    int ix[ORDER + 1], iy[ORDER + 1], iz[ORDER + 1];
#pragma unroll
                    for (int k = 0; k <= ORDER; ++k) {
                        ix[k] = mirror_idx(t0[0] + k, nx);
                        iy[k] = ny - 1 - mirror_idx(t0[1] + k, ny);
                        iz[k] = mirror_idx(t0[2] + k, nz);
                    }
#pragma unroll
                    for (int k2 = 0; k2 <= ORDER; ++k2) {
#pragma unroll
                        for (int k0 = 0; k0 <= ORDER; ++k0) {
                            const int col = (iz[k2] * nx + ix[k0]) * yp;
                            float2 r = make_float2(0.f, 0.f);
#pragma unroll
                            for (int k1 = 0; k1 <= ORDER; ++k1)
                                r = ffma2(make_float2(wt[1][k1], wt[1][k1]), __ldg(sa + (col + iy[k1])), r);
                            const float w02 = wt[2][k2] * wt[0][k0];
                            acc = ffma2(make_float2(w02, w02), r, acc);
                        }
                    }
                }
                part[q] = acc;
            }
            if ((a % R3_KAHAN) == R3_KAHAN - 1 || a == nb - 1) {
#pragma unroll
                for (int q = 0; q < R3_Z; ++q) {
                    kahan_add(s[q], cp[q], part[q]);
                    part[q] = make_float2(0.f, 0.f);
                }
            }
        }
    }
    if (vxy) {
#pragma unroll
        for (int q = 0; q < R3_Z; ++q) {
            const int z = z0 + q;
            if (z < nz)
                store_sum<ONLYREAL>(R, volume, comp, ((size_t)z * ny + y) * nx + x, s[q], cp[q]);
        }
    }
}

// cuTensorMapEncodeTiled from the driver, looked up once through the
// runtime (no link-time dependency on libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// Tensor maps of a batch's y-axis slab [a][z][x][ypitch] (8-byte
// elements), one per TMA box shape [zb][xb][Y y].
template <int ORDER>
static cudaError_t encode_slab_maps(const RotParams &R, const float2 *slab, RotMaps &maps)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc)
        return cudaErrorNotSupported;
    const cuuint64_t dims[4] = {(cuuint64_t)R.ypitch, (cuuint64_t)R.nx, (cuuint64_t)R.nz,
                                (cuuint64_t)R.nbatch_angles};
    const cuuint64_t strides[3] = {(cuuint64_t)R.ypitch * 8, (cuuint64_t)R.nx * R.ypitch * 8,
                                   (cuuint64_t)R.nz * R.nx * R.ypitch * 8};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    for (int iz = 0; iz < R2_NTMA; ++iz)
        for (int ix = 0; ix < R2_NTMA; ++ix) {
            const cuuint32_t boxd[4] = {(cuuint32_t)RotY<ORDER>::Y, (cuuint32_t)r2_tma_box<ORDER>(ix),
                                        (cuuint32_t)r2_tma_box<ORDER>(iz), 1};
            const CUresult r = enc(&maps.m[iz * R2_NTMA + ix], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4,
                                   const_cast<float2 *>(slab), dims, strides, boxd, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS)
                return cudaErrorInvalidValue;
        }
    return cudaSuccess;
}

// The TMA path needs slab rows of Y y that start on 16-byte boundaries and
// 16-byte aligned strides (a y pitch that is a multiple of Y) and a 16-byte
// aligned slab.
template <int ORDER>
static bool rotate_tma_ok(const RotParams &R, const float2 *slab)
{
    return kRotateTma && R.ypitch % RotY<ORDER>::Y == 0 && ((uintptr_t)slab % 16) == 0 &&
           tensor_map_encoder() != nullptr;
}

template <int ORDER, bool ONLYREAL>
static cudaError_t rotate_impl(const RotParams &R, int tilted, const float2 *slab, const double *geo, void *volume,
                               float2 *comp, void *scratch, cudaStream_t s)
{
    if (!tilted) {
        const int ntiles = ((R.nx + R2_T - 1) / R2_T) * ((R.nz + R2_T - 1) / R2_T);
        const int nset = R.nbatch_angles * ntiles;
        TileGeo *tiles = reinterpret_cast<TileGeo *>(scratch);
        if (R.ny == 1 && R.ypitch == 1) {
            k_rotate_y_setup<ORDER, false><<<(nset + 127) / 128, 128, 0, s>>>(R, geo, tiles);
            dim3 grid((R.nx + R2_T - 1) / R2_T, (R.nz + R2_T - 1) / R2_T);
            k_rotate_plane<ORDER, ONLYREAL><<<grid, R2_T * R2_T, 0, s>>>(R, slab, geo, tiles, volume, comp);
        } else {
            constexpr int Y = RotY<ORDER>::Y;
            dim3 grid((R.nx + R2_T - 1) / R2_T, (R.nz + R2_T - 1) / R2_T, (R.ny + Y - 1) / Y);
            RotMaps maps;
            std::memset(&maps, 0, sizeof maps);
            if (rotate_tma_ok<ORDER>(R, slab) && encode_slab_maps<ORDER>(R, slab, maps) == cudaSuccess) {
                k_rotate_y_setup<ORDER, true><<<(nset + 127) / 128, 128, 0, s>>>(R, geo, tiles);
                k_rotate_y<ORDER, ONLYREAL, true>
                    <<<grid, R2_THREADS, RotY<ORDER>::SMEM, s>>>(R, slab, geo, tiles, volume, comp, maps);
            } else {
                k_rotate_y_setup<ORDER, false><<<(nset + 127) / 128, 128, 0, s>>>(R, geo, tiles);
                k_rotate_y<ORDER, ONLYREAL, false>
                    <<<grid, R2_THREADS, RotY<ORDER>::SMEM, s>>>(R, slab, geo, tiles, volume, comp, maps);
            }
        }
    } else {
        dim3 grid((R.nx + R3_X - 1) / R3_X, (R.ny + R3_Y - 1) / R3_Y, (R.nz + R3_Z - 1) / R3_Z);
        k_rotate_3d<ORDER, ONLYREAL><<<grid, R3_X * 32, 0, s>>>(R, slab, geo, volume, comp);
    }
    return cudaGetLastError();
}

size_t rotate_scratch_bytes(int nbatch_angles, int ny, int nx, int nz, int tilted)
{
    (void)ny;
    if (tilted)
        return 0;
    const size_t ntiles = (size_t)((nx + R2_T - 1) / R2_T) * ((nz + R2_T - 1) / R2_T);
    return (size_t)nbatch_angles * ntiles * sizeof(TileGeo);
}

template <int ORDER>
static cudaError_t configure_rotate_order()
{
    const void *fns[] = {(const void *)k_rotate_y<ORDER, false, false>, (const void *)k_rotate_y<ORDER, true, false>,
                         (const void *)k_rotate_y<ORDER, false, true>, (const void *)k_rotate_y<ORDER, true, true>};
    for (const void *f : fns) {
        const cudaError_t e =
            cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RotY<ORDER>::SMEM);
        if (e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

cudaError_t configure_rotate_kernels()
{
    cudaError_t e;
    if ((e = configure_rotate_order<0>()) || (e = configure_rotate_order<1>()) ||
        (e = configure_rotate_order<2>()) || (e = configure_rotate_order<3>()) ||
        (e = configure_rotate_order<4>()) || (e = configure_rotate_order<5>()))
        return e;
    return cudaSuccess;
}

cudaError_t launch_rotate(const RotParams &R, int order, int tilted, const float2 *slab, const double *geo,
                          void *volume, float2 *comp, void *scratch, cudaStream_t s)
{
#define ODT_ROT_CASE(O)                                                                       \
    case O:                                                                                   \
        return R.onlyreal ? rotate_impl<O, true>(R, tilted, slab, geo, volume, comp, scratch, s) \
                          : rotate_impl<O, false>(R, tilted, slab, geo, volume, comp, scratch, s);
    switch (order) {
        ODT_ROT_CASE(0)
        ODT_ROT_CASE(1)
        ODT_ROT_CASE(2)
        ODT_ROT_CASE(3)
        ODT_ROT_CASE(4)
        ODT_ROT_CASE(5)
    default:
        return cudaErrorInvalidValue;
    }
#undef ODT_ROT_CASE
}

// ---------------------------------------------------------------------------
// Transpose of the y-axis resampling (the backward pass):
//   slab_grad[a][y][iz][ix] = sum over outputs o of angle a whose taps
//       (mirrored) include (iz, ix): wz * wx * vol_grad[o_z][y][o_x]
// with exactly the forward's in/out decisions, tap starts and weights.
//
// Work split (the transpose of k_rotate_y): a CTA owns a 16 x 16 tile of
// coefficients (iz, ix) and 16 y (the lanes of a half-warp) and loops over
// the batch's angles.  Per angle, k_rotate_y_adj_setup has found the box of
// outputs whose coordinates come within reach of the tile's (virtual, for
// mirrored edges) tap positions; one thread per output computes its
// parameter record (in/out decision, tap start, weights) into shared memory,
// then every half-warp pushes w * g of its outputs' taps that land in the
// tile into a shared accumulator with shared-memory atomics (the 16 lanes
// are 16 different y, so one instruction never collides with itself).  The
// tile is written once per angle.
constexpr int RA_T = 16, RA_Y = 16, RA_THREADS = 512;
constexpr int RA_OBOX = 36;        // max output box per axis
constexpr int RA_YP = RA_Y + 1;    // accumulator y pitch (conflict-free reads)
constexpr size_t RA_SMEM = (size_t)RA_T * RA_T * RA_YP * sizeof(float2) + (size_t)RA_OBOX * RA_OBOX * 8 * sizeof(float);

struct __align__(16) AdjTileGeo {
    AxisCoord z, x;              // coordinates of output (oz0, ox0)
    short oz0, ox0, ozn, oxn;    // box of candidate outputs; ozn == 0: none
    short vz0, vz1, vx0, vx1;    // virtual tap range that can land in the tile
};
static_assert(sizeof(AdjTileGeo) == 64, "AdjTileGeo is one 64-byte record");

// Virtual tap range [v0, v1] whose mirror images can fall in the real range
// [t0, t1] of an axis of length n (taps reach at most two positions past
// either edge for orders <= 3).
__device__ __forceinline__ void virtual_range(int t0, int t1, int n, int &v0, int &v1)
{
    v0 = t0;
    v1 = t1;
    if (t0 <= 2)
        v0 = -2;
    if (t1 >= n - 3)
        v1 = n + 1;
}

template <int ORDER>
__global__ void k_rotate_y_adj_setup(RotParams R, const double *__restrict__ geo, AdjTileGeo *__restrict__ tiles)
{
    const int ntz = (R.nz + RA_T - 1) / RA_T, ntx = (R.nx + RA_T - 1) / RA_T;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= R.nbatch_angles * ntz * ntx)
        return;
    const int a = id / (ntz * ntx), t = id % (ntz * ntx);
    const int cz0 = (t / ntx) * RA_T, cx0 = (t % ntx) * RA_T;
    const int nz = R.nz, nx = R.nx;
    const double *g = geo + 6 * (size_t)a;
    const double m00 = g[0], m01 = g[1], m10 = g[2], m11 = g[3], f0 = g[4], f1 = g[5];
    int vz0, vz1, vx0, vx1;
    virtual_range(cz0, min(cz0 + RA_T, nz) - 1, nz, vz0, vz1);
    virtual_range(cx0, min(cx0 + RA_T, nx) - 1, nx, vx0, vx1);
    AdjTileGeo tg;
    tg.vz0 = (short)vz0;
    tg.vz1 = (short)vz1;
    tg.vx0 = (short)vx0;
    tg.vx1 = (short)vx1;
    tg.oz0 = tg.ox0 = tg.ozn = tg.oxn = 0;
    // outputs whose taps can reach the virtual range have coordinates within
    // 2.5 of it (tap windows are at most 4 wide), and inside [0, n-1]
    const double czl = fmax((double)vz0 - 2.5, 0.0), czh = fmin((double)vz1 + 2.5, (double)(nz - 1));
    const double cxl = fmax((double)vx0 - 2.5, 0.0), cxh = fmin((double)vx1 + 2.5, (double)(nx - 1));
    // o = M^T (c - f) (M is a rotation)
    double ozl = 1e30, ozh = -1e30, oxl = 1e30, oxh = -1e30;
    for (int k = 0; k < 4; ++k) {
        const double cz = (k & 1) ? czh : czl, cx = (k & 2) ? cxh : cxl;
        const double oz = m00 * (cz - f0) + m10 * (cx - f1), ox = m01 * (cz - f0) + m11 * (cx - f1);
        ozl = fmin(ozl, oz);
        ozh = fmax(ozh, oz);
        oxl = fmin(oxl, ox);
        oxh = fmax(oxh, ox);
    }
    const int oz0 = max(0, (int)floor(ozl) - 1), oz1 = min(nz - 1, (int)ceil(ozh) + 1);
    const int ox0 = max(0, (int)floor(oxl) - 1), ox1 = min(nx - 1, (int)ceil(oxh) + 1);
    if (oz0 <= oz1 && ox0 <= ox1) {
        if (oz1 - oz0 + 1 > RA_OBOX || ox1 - ox0 + 1 > RA_OBOX) {
            atomicOr(R.status, DEVCHK_BOX_OVERFLOW);
        } else {
            tg.oz0 = (short)oz0;
            tg.ox0 = (short)ox0;
            tg.ozn = (short)(oz1 - oz0 + 1);
            tg.oxn = (short)(ox1 - ox0 + 1);
        }
    }
    tg.z = make_axis((f0 + m00 * (double)tg.oz0) + m01 * (double)tg.ox0, m00, m01);
    tg.x = make_axis((f1 + m10 * (double)tg.oz0) + m11 * (double)tg.ox0, m10, m11);
    tiles[id] = tg;
}

template <int ORDER>
__global__ void __launch_bounds__(RA_THREADS, 2) k_rotate_y_adjoint(RotParams R, const float2 *__restrict__ vgrad,
                                                                    const double *__restrict__ geo,
                                                                    const AdjTileGeo *__restrict__ tiles,
                                                                    float2 *__restrict__ sgrad)
{
    extern __shared__ float4 ra_smem[];
    // accumulators [16 z][16 x][RA_YP], real and imaginary parts in separate
    // planes (the 16 lanes of an output add into 16 consecutive words, so the
    // two outputs of a warp do not meet on the same even banks)
    float *acc_re = reinterpret_cast<float *>(ra_smem);
    float *acc_im = acc_re + RA_T * RA_T * RA_YP;
    float4 *rec = reinterpret_cast<float4 *>(acc_im + RA_T * RA_T * RA_YP);  // [box][2]
    const int tid = threadIdx.x, hw = tid >> 4, yl = tid & 15;
    const int nx = R.nx, nz = R.nz, ny = R.ny;
    const int ntx = (nx + RA_T - 1) / RA_T, ntz = (nz + RA_T - 1) / RA_T;
    const int tile = blockIdx.y * ntx + blockIdx.x;
    const int cx0 = blockIdx.x * RA_T, cz0 = blockIdx.y * RA_T, y0 = blockIdx.z * RA_Y;
    const int y = y0 + yl;
    const bool yok = y < ny;
    for (int a = 0; a < R.nbatch_angles; ++a) {
        const AdjTileGeo tg = tiles[(size_t)a * ntz * ntx + tile];
        for (int i = tid; i < RA_T * RA_T * RA_YP; i += RA_THREADS) {
            acc_re[i] = 0.f;
            acc_im[i] = 0.f;
        }
        const int nbox = tg.ozn * tg.oxn;
        const double *g = geo + 6 * (size_t)a;
        // parameter records: (pz, px, wz0, wz1) (wz2, wx0, wx1, wx2), where
        // byte i of pz (px) is the tile-relative position of z (x) tap i
        // after mirroring, 0xFF for a tap outside the tile; pz = -1 when the
        // output is outside the domain or none of its taps lands in the tile
        for (int o = tid; o < nbox; o += RA_THREADS) {
            const int dz = o / tg.oxn, dx = o - dz * tg.oxn;
            const int oz = tg.oz0 + dz, ox = tg.ox0 + dx;
            int Iz, Ix;
            const float lz = eval_axis(tg.z, (float)dz, (float)dx, Iz);
            const float lx = eval_axis(tg.x, (float)dz, (float)dx, Ix);
            bool in = inside_axis(lz, Iz, nz, [&] {
                return __dadd_rn(__dadd_rn(__ldg(g + 4), __dmul_rn(__ldg(g + 0), (double)oz)),
                                 __dmul_rn(__ldg(g + 1), (double)ox));
            });
            in = in && inside_axis(lx, Ix, nx, [&] {
                return __dadd_rn(__dadd_rn(__ldg(g + 5), __dmul_rn(__ldg(g + 2), (double)oz)),
                                 __dmul_rn(__ldg(g + 3), (double)ox));
            });
            int pz = -1, px = -1;
            float wz[4] = {0.f, 0.f, 0.f, 0.f}, wx[4] = {0.f, 0.f, 0.f, 0.f};
            if (in) {
                int sz, sx;
                if (ORDER == 0) {
                    const double cz = __dadd_rn(__dadd_rn(__ldg(g + 4), __dmul_rn(__ldg(g + 0), (double)oz)),
                                                __dmul_rn(__ldg(g + 1), (double)ox));
                    const double cx = __dadd_rn(__dadd_rn(__ldg(g + 5), __dmul_rn(__ldg(g + 2), (double)oz)),
                                                __dmul_rn(__ldg(g + 3), (double)ox));
                    sz = (int)floor(cz + 0.5);
                    sx = (int)floor(cx + 0.5);
                    wz[0] = 1.f;
                    wx[0] = 1.f;
                } else {
                    float w[ORDER + 1];
                    sz = Iz + Spline<ORDER>::weights(lz, w);
#pragma unroll
                    for (int k = 0; k <= ORDER; ++k)
                        wz[k] = w[k];
                    sx = Ix + Spline<ORDER>::weights(lx, w);
#pragma unroll
                    for (int k = 0; k <= ORDER; ++k)
                        wx[k] = w[k];
                }
                if (sz + ORDER >= tg.vz0 && sz <= tg.vz1 && sx + ORDER >= tg.vx0 && sx <= tg.vx1) {
                    bool anyz = false, anyx = false;
                    unsigned uz = 0xFFFFFFFFu, ux = 0xFFFFFFFFu;
#pragma unroll
                    for (int i = 0; i <= ORDER; ++i) {
                        const int zz = mirror_idx(sz + i, nz) - cz0, xx = mirror_idx(sx + i, nx) - cx0;
                        const bool zin = zz >= 0 && zz < RA_T, xin = xx >= 0 && xx < RA_T;
                        const unsigned sh = 8u * (unsigned)i;
                        uz = (uz & ~(0xFFu << sh)) | ((zin ? (unsigned)zz : 0xFFu) << sh);
                        ux = (ux & ~(0xFFu << sh)) | ((xin ? (unsigned)xx : 0xFFu) << sh);
                        anyz = anyz || zin;
                        anyx = anyx || xin;
                    }
                    pz = (anyz && anyx) ? (int)uz : -1;
                    px = (int)ux;
                }
            }
            rec[2 * o] = make_float4(__int_as_float(pz), __int_as_float(px), wz[0], wz[1]);
            rec[2 * o + 1] = make_float4(wz[2], wx[0], wx[1], wx[2]);
            if (ORDER == 3) {
                // order 3 needs wz[3], wx[3]: the box holds at most
                // RA_OBOX^2 records of 8 words; keep the fourth weights in
                // the high half of the record array
                float2 *w4 = reinterpret_cast<float2 *>(rec + 2 * RA_OBOX * RA_OBOX);
                w4[o] = make_float2(wz[3], wx[3]);
            }
        }
        __syncthreads();
        // push: half-warp hw takes outputs hw, hw + 32, ...
        for (int o = hw; o < nbox; o += RA_THREADS / 16) {
            const float4 r0 = rec[2 * o];
            const int pz = __float_as_int(r0.x);
            if (pz == -1)
                continue;
            const float4 r1 = rec[2 * o + 1];
            const unsigned upz = (unsigned)pz, upx = (unsigned)__float_as_int(r0.y);
            float wz[4] = {r0.z, r0.w, r1.x, 0.f}, wx[4] = {r1.y, r1.z, r1.w, 0.f};
            if (ORDER == 3) {
                const float2 w4 = reinterpret_cast<const float2 *>(rec + 2 * RA_OBOX * RA_OBOX)[o];
                wz[3] = w4.x;
                wx[3] = w4.y;
            }
            const int dz = o / tg.oxn, dx = o - dz * tg.oxn;
            const int oz = tg.oz0 + dz, ox = tg.ox0 + dx;
            // vgrad is the volume gradient in the [z][x][y] order: the 16
            // lanes (consecutive y) of an output read one 128-byte run
            const float2 gv = yok ? __ldg(vgrad + ((size_t)oz * nx + ox) * ny + y) : make_float2(0.f, 0.f);
#pragma unroll
            for (int i = 0; i <= ORDER; ++i) {
                const int zz = (int)((upz >> (8 * i)) & 0xFFu);
                if (zz == 0xFF)
                    continue;
#pragma unroll
                for (int k = 0; k <= ORDER; ++k) {
                    const int xx = (int)((upx >> (8 * k)) & 0xFFu);
                    if (xx == 0xFF)
                        continue;
                    const float w = wz[i] * wx[k];
                    const int idx = (zz * RA_T + xx) * RA_YP + yl;
                    atomicAdd(acc_re + idx, w * gv.x);
                    atomicAdd(acc_im + idx, w * gv.y);
                }
            }
        }
        __syncthreads();
        // write the tile: slab_grad[a][y][z][x], runs of 16 x
        for (int e = tid; e < RA_T * RA_T * RA_Y; e += RA_THREADS) {
            const int xx = e & 15, zz = (e >> 4) & 15, yy = e >> 8;
            const int z = cz0 + zz, x = cx0 + xx, yv = y0 + yy;
            const int idx = (zz * RA_T + xx) * RA_YP + yy;
            if (z < nz && x < nx && yv < ny)
                sgrad[(((size_t)a * ny + yv) * nz + z) * nx + x] = make_float2(acc_re[idx], acc_im[idx]);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Transpose of the tilted resampling (k_rotate_3d):
//   slab_grad[a][Z][X][Y] += sum over outputs o of angle a whose (mirrored)
//       taps include (Z, X, Y) of w0 w1 w2 * vol_grad[o]
// in the forward's slab layout [a][z][x][y] (pitch R.ypitch).  The tiles,
// FP32 coordinates, in/out decisions (FP64 re-evaluation near the domain
// edge), tap starts and weights are those of k_rotate_3d, so this is the
// exact transpose of the forward's arithmetic.  Each output pushes its
// (ORDER+1)^3 taps with global atomic adds; the 32 lanes of a warp are
// consecutive y, whose taps fall on nearly consecutive slab y, so a warp's
// adds hit one or two 256-byte runs.  slab_grad must start at zero.
template <int ORDER>
__global__ void __launch_bounds__(256, ORDER >= 4 ? 2 : 4) k_rotate_3d_adjoint(RotParams R,
                                                                            const float2 *__restrict__ vol_grad,
                                                                            const double *__restrict__ geo,
                                                                            float2 *slab_grad)
{
    __shared__ AxisCoord3 srec[R3_CHUNK][3];
    __shared__ int sflag[R3_CHUNK][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nx = R.nx, ny = R.ny, nz = R.nz, yp = R.ypitch;
    const int x0 = blockIdx.x * R3_X, y0 = blockIdx.y * R3_Y, z0 = blockIdx.z * R3_Z;
    const int x = x0 + w, y = y0 + lane;
    const bool vxy = x < nx && y < ny;
    const bool full = x0 + R3_X <= nx && y0 + R3_Y <= ny && z0 + R3_Z <= nz;
    const int n3[3] = {nx, ny, nz};
    const size_t aslab = (size_t)nz * nx * yp;
    const float d0 = (float)w, d1 = (float)(-lane);
    const double o0 = (double)x, o1 = (double)(ny - 1 - y);
    float2 gv[R3_Z];
#pragma unroll
    for (int q = 0; q < R3_Z; ++q) {
        const int z = z0 + q;
        gv[q] = (vxy && z < nz) ? __ldg(vol_grad + ((size_t)z * ny + y) * nx + x) : make_float2(0.f, 0.f);
    }
    const int nb = R.nbatch_angles;
    for (int a0 = 0; a0 < nb; a0 += R3_CHUNK) {
        const int na = min(R3_CHUNK, nb - a0);
        __syncthreads();
        for (int t = threadIdx.x; t < na * 3; t += blockDim.x) {
            const int aa = t / 3, i = t % 3;
            const double *g = geo + 12 * (size_t)(a0 + aa);
            const double m0 = g[3 * i], m1 = g[3 * i + 1], m2 = g[3 * i + 2];
            const double c = ((g[9 + i] + m0 * (double)x0) + m1 * (double)(ny - 1 - y0)) + m2 * (double)z0;
            srec[aa][i] = make_axis3(c, m0, m1, m2);
            const double e0 = m0 * (R3_X - 1), e1 = -m1 * (R3_Y - 1), e2 = m2 * (R3_Z - 1);
            const double lo = c + fmin(e0, 0.0) + fmin(e1, 0.0) + fmin(e2, 0.0);
            const double hi = c + fmax(e0, 0.0) + fmax(e1, 0.0) + fmax(e2, 0.0);
            sflag[aa][i] = (full && lo >= R3_LO<ORDER> && hi <= n3[i] - R3_HI<ORDER>) ? 1 : 0;
        }
        __syncthreads();
        for (int aa = 0; aa < na; ++aa) {
            const int a = a0 + aa;
            const bool interior = sflag[aa][0] && sflag[aa][1] && sflag[aa][2];
            const AxisCoord3 *axp = srec[aa];
            float2 *sg = slab_grad + (size_t)a * aslab;
            const double *g = geo + 12 * (size_t)a;
#pragma unroll
            for (int q = 0; q < R3_Z; ++q) {
                const int z = z0 + q;
                if (!vxy || z >= nz)
                    continue;
                const float d2 = (float)q;
                int Ib[3];
                float l[3];
                l[0] = eval_axis3(axp[0], d0, d1, d2, Ib[0]);
                l[1] = eval_axis3(axp[1], d0, d1, d2, Ib[1]);
                l[2] = eval_axis3(axp[2], d0, d1, d2, Ib[2]);
                const double o2 = (double)z;
                auto exact = [&](int i) {
                    return __dadd_rn(__dadd_rn(__dadd_rn(__ldg(g + 9 + i), __dmul_rn(__ldg(g + 3 * i), o0)),
                                               __dmul_rn(__ldg(g + 3 * i + 1), o1)),
                                     __dmul_rn(__ldg(g + 3 * i + 2), o2));
                };
                if (!interior) {
                    bool in = true;
#pragma unroll
                    for (int i = 0; i < 3; ++i)
                        in = in && inside_axis(l[i], Ib[i], n3[i], [&] { return exact(i); });
                    if (!in)
                        continue;
                }
                int t0[3];
                float wt[3][ORDER + 1];
                if (ORDER == 0) {
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        t0[i] = (int)floor(exact(i) + 0.5);
                        wt[i][0] = 1.f;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 3; ++i)
                        t0[i] = Ib[i] + Spline<ORDER>::weights(l[i], wt[i]);
                }
                int ix[ORDER + 1], iy[ORDER + 1], iz[ORDER + 1];
#pragma unroll
                for (int k = 0; k <= ORDER; ++k) {
                    ix[k] = interior ? t0[0] + k : mirror_idx(t0[0] + k, nx);
                    iy[k] = ny - 1 - (interior ? t0[1] + k : mirror_idx(t0[1] + k, ny));
                    iz[k] = interior ? t0[2] + k : mirror_idx(t0[2] + k, nz);
                }
                const float2 gq = gv[q];
#pragma unroll
                for (int k2 = 0; k2 <= ORDER; ++k2) {
#pragma unroll
                    for (int k0 = 0; k0 <= ORDER; ++k0) {
                        float2 *col = sg + ((size_t)iz[k2] * nx + ix[k0]) * yp;
                        const float w02 = wt[2][k2] * wt[0][k0];
#pragma unroll
                        for (int k1 = 0; k1 <= ORDER; ++k1) {
                            const float wv = w02 * wt[1][k1];
                            atomicAdd(&col[iy[k1]].x, wv * gq.x);
                            atomicAdd(&col[iy[k1]].y, wv * gq.y);
                        }
                    }
                }
            }
        }
    }
}

cudaError_t launch_rotate_adjoint(const RotParams &R, int order, int tilted, const float2 *vol_grad,
                                  const double *geo, float2 *slab_grad, void *scratch, cudaStream_t s)
{
    if (tilted) {
        // slab_grad accumulates atomically: cleared first (stream-ordered)
        cudaError_t e =
            cudaMemsetAsync(slab_grad, 0, (size_t)R.nbatch_angles * R.nz * R.nx * R.ypitch * sizeof(float2), s);
        if (e != cudaSuccess)
            return e;
        dim3 grid((R.nx + R3_X - 1) / R3_X, (R.ny + R3_Y - 1) / R3_Y, (R.nz + R3_Z - 1) / R3_Z);
        switch (order) {
#define ODT_ADJ3_CASE(O)                                                              \
    case O:                                                                           \
        k_rotate_3d_adjoint<O><<<grid, R3_X * 32, 0, s>>>(R, vol_grad, geo, slab_grad); \
        break;
            ODT_ADJ3_CASE(0)
            ODT_ADJ3_CASE(1)
            ODT_ADJ3_CASE(2)
            ODT_ADJ3_CASE(3)
#undef ODT_ADJ3_CASE
        default:
            return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    const int ntiles = ((R.nx + RA_T - 1) / RA_T) * ((R.nz + RA_T - 1) / RA_T);
    const int nset = R.nbatch_angles * ntiles;
    AdjTileGeo *tiles = reinterpret_cast<AdjTileGeo *>(scratch);
    dim3 grid((R.nx + RA_T - 1) / RA_T, (R.nz + RA_T - 1) / RA_T, (R.ny + RA_Y - 1) / RA_Y);
    const size_t smem = RA_SMEM + (size_t)RA_OBOX * RA_OBOX * sizeof(float2);
    switch (order) {
#define ODT_ADJ_CASE(O)                                                                                      \
    case O:                                                                                                  \
        k_rotate_y_adj_setup<O><<<(nset + 127) / 128, 128, 0, s>>>(R, geo, tiles);                          \
        k_rotate_y_adjoint<O><<<grid, RA_THREADS, smem, s>>>(R, vol_grad, geo, tiles, slab_grad);           \
        break;
        ODT_ADJ_CASE(0)
        ODT_ADJ_CASE(1)
        ODT_ADJ_CASE(2)
        ODT_ADJ_CASE(3)
#undef ODT_ADJ_CASE
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// [z][y][x] -> [z][x][y], 32 x 32 tiles of one z plane through shared
// memory (coalesced reads along x, writes along y).
__global__ void __launch_bounds__(256) k_volume_zxy(const float2 *__restrict__ src, float2 *__restrict__ dst, int ny,
                                                    int nx)
{
    __shared__ float2 t[32][33];
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32, z = blockIdx.z;
    const size_t plane = (size_t)z * ny * nx;
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int y = y0 + i, x = x0 + threadIdx.x;
        if (y < ny && x < nx)
            t[i][threadIdx.x] = src[plane + (size_t)y * nx + x];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int x = x0 + i, y = y0 + threadIdx.x;
        if (x < nx && y < ny)
            dst[plane + (size_t)x * ny + y] = t[threadIdx.x][i];
    }
}

cudaError_t launch_volume_zxy(const float2 *vol, float2 *vol_zxy, int nz, int ny, int nx, cudaStream_t s)
{
    dim3 grid((nx + 31) / 32, (ny + 31) / 32, nz);
    k_volume_zxy<<<grid, dim3(32, 8), 0, s>>>(vol, vol_zxy, ny, nx);
    return cudaGetLastError();
}

cudaError_t configure_rotate_adjoint_kernels()
{
    const size_t smem = RA_SMEM + (size_t)RA_OBOX * RA_OBOX * sizeof(float2);
    const void *fns[] = {(const void *)k_rotate_y_adjoint<0>, (const void *)k_rotate_y_adjoint<1>,
                         (const void *)k_rotate_y_adjoint<2>, (const void *)k_rotate_y_adjoint<3>};
    for (const void *f : fns) {
        const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

}  // namespace odt
