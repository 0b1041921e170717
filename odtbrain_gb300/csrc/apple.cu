// Missing-apple-core correction on the GPU: odtbrain.apple.correct
// (odtbrain/apple.py:113-263) with apple_core_3d (:8-53), the constraints
// constraint_nn / constraint_sh (:56-110), envelope_gauss (:289-350) and
// spillover_region / ellipsoid_shell (:281-286, 353-363).
//
// The volume (n0, n1, n2) = (Nx, Ny, Nx) stays in HBM as complex64; the
// 3D FFTs (single precision, unnormalised, like the reference's pyFFTW
// plans) are line transforms in registers (odt_fft.cuh), one kernel per
// axis.  One iteration of the reference's loop is five kernels:
//   k_apple_s (axis 1, forward)
//   k_apple_s (axis 0, forward; then per voxel: envelope suppression,
//              DC update (method "sh"), restore of the non-core spectrum,
//              sum of |spectrum| over the core; then axis 0 inverse)
//   k_apple_dec  stopping criterion, one thread, in float32 like the
//              reference's NumPy scalars
//   k_apple_s (axis 1, inverse)
//   k_apple_x (axis 2 inverse, times fl32(1/N) -> result; for "nn" and a
//              following iteration also the constraint and the axis 2
//              forward transform of the next iteration)
// Kernels of iterations after the stop return at once; the host enqueues
// iterations in chunks and reads the stop word between chunks.  Method
// "sh" needs the spatial histogram before its constraint: per iteration
// k_sh_minmax, k_sh_hist (NumPy's bin assignment), and the host computes
// the thresholds from the 100 counts exactly as the reference's NumPy code.
//
// Once per call: voxel flags (core, spillover, background shell, user mask)
// from the reference's FP64 formulas (k_apple_flags), the initial forward
// transform (the original spectrum), and the envelope: |spectrum| with the
// core set to NaN, padded and fftshifted (k_env_pad), the core filled from
// the x/y-swapped volume (k_env_swap), remaining NaNs from the nearest known
// voxel (Maurer et al.'s exact Euclidean feature transform, the algorithm
// scipy.ndimage.distance_transform_edt implements: k_edt_*), and scipy's
// gaussian_filter (FP64 sums in its order, float32 after each axis,
// k_env_gauss).
//
// The same kernels serve constraint_nn / constraint_sh and envelope_gauss
// called on their own (odt_apple_constrain, odt_apple_envelope), for
// float32 or float64 data: k_sh_minmax / k_sh_hist / k_constrain and the
// envelope pipeline, templated on the data's type.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/odtbrain_gb300.h"
#include "odt_fft.cuh"
#include "odt_internal.cuh"
#include "odt_stage_util.cuh"

namespace odt {
namespace {

constexpr uint8_t F_CORE = 1, F_SPOV = 2, F_SHELL = 4, F_MASK = 8;
constexpr int CHUNK = 8;      // iterations enqueued between stop checks
constexpr int HIST_BINS = 100;

struct AppleCtl {
    float prev, norm;
    int stop;   // iterations done when the loop stopped, 0 while running
    int iters;  // iterations done
    unsigned long long minkey, maxkey;  // ordered keys (method "sh")
    float lo, hi, fmin, fmax;           // method "sh" thresholds
    unsigned int nan_count;
    unsigned int pad;
};

struct AP {
    int n0, n1, n2;
    long long N;
    const float2 *tw0, *tw1, *tw2;
    const uint8_t *flags;
    const float *evlp;  // NULL: envelope off
    float ee;
    float2 *orig;
    float2 *buf;
    float2 *data;
    const float *freal;
    double *state;  // [max_iter + 1], FP64 sums of |spectrum| over the core
    AppleCtl *ctl;
    int method;  // 0 nn, 1 sh, 2 none
    int max_iter;
    float min_diff;
    float scale;
    int has_mask;
    unsigned int *hist;  // [HIST_BINS] (method "sh")
    const float *edges;  // [HIST_BINS + 1] (method "sh")
};

__device__ __forceinline__ bool ran_out(const AP &P, int it)
{
    const int s = *(volatile const int *)&P.ctl->stop;
    return s != 0 && s <= it;
}

// The real part after one spatial constraint (the imaginary part becomes 0):
// method 0 constraint_nn (apple.py:56-72), 1 constraint_sh (apple.py:75-110)
// with the thresholds fmin, fmax (over the spillover region and shell) and
// lo, hi (the histogram's half-maximum bin centres).  Halving is exact.
template <typename T>
__device__ __forceinline__ T constrain_re(int method, bool has_mask, T re, uint8_t fl, T fmin, T fmax, T lo, T hi)
{
    if (method == 0) {
        if (fl & F_SHELL)
            re = T(0);
        if (fl & F_SPOV)
            re = T(0);
        bool low = re < T(0);
        if (has_mask)
            low = low && (fl & F_MASK);
        if (low)
            re = T(0);
    } else {
        const bool below = re > fmin && re < lo;
        const bool above = re > hi && re < fmax;
        bool out = below || above;
        if (has_mask)
            out = out && (fl & F_MASK);
        if (out)
            re = re * T(0.5);
        if (fl & F_SHELL)
            re = re * T(0.5);
    }
    return re;
}

// Spatial constraint of the reference's loop on one voxel value.
__device__ __forceinline__ float2 constrain(const AP &P, float2 d, uint8_t fl, float fmin, float fmax, float lo,
                                            float hi)
{
    if (P.method == 2)  // neither constraint (apple.py:222-227 with another method)
        return d;
    return make_float2(constrain_re<float>(P.method, P.has_mask, d.x, fl, fmin, fmax, lo, hi), 0.f);
}

// ---- axis 2 (contiguous lines) --------------------------------------------
// mode 0: f.real -> forward -> buf (the original spectrum's first axis)
// mode 1: constrain(f.real) -> forward -> buf (iteration 0's first axis)
// mode 2: buf -> inverse -> * scale -> data; for "nn" with a following
//         iteration: constrain -> forward -> buf
// mode 3: constrain(data) -> forward -> buf (method "sh")
template <class L, int LPC>
__global__ void __launch_bounds__(LPC *L::TPL) k_apple_x(AP P, L line, int mode, int it)
{
    if (mode >= 2 && ran_out(P, it))
        return;
    extern __shared__ float2 smem[];
    const int n = line.size();
    const int ls = xslots<false>(n);
    float2 *buf0 = smem, *buf1 = smem + LPC * ls, *tw = smem + 2 * LPC * ls;
    copy_twiddles<L>(tw, P.tw2, n);
    const int l = threadIdx.x / L::TPL, j = threadIdx.x % L::TPL;
    const long long lid = (long long)blockIdx.x * LPC + l;
    const bool valid = lid < (long long)P.n0 * P.n1;
    const long long base = valid ? lid * n : 0;
    float fmin = 0.f, fmax = 0.f, lo = 0.f, hi = 0.f;
    if (P.method == 1) {
        fmin = P.ctl->fmin;
        fmax = P.ctl->fmax;
        lo = P.ctl->lo;
        hi = P.ctl->hi;
    }
    float2 v[L::SLOTS];
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int x = j + r * L::TPL;
        float2 a = make_float2(0.f, 0.f);
        if (valid && x < n) {
            if (mode <= 1)
                a = make_float2(P.freal[base + x], 0.f);
            else if (mode == 2)
                a = P.buf[base + x];
            else
                a = P.data[base + x];
            if (mode == 1 || mode == 3)
                a = constrain(P, a, P.flags[base + x], fmin, fmax, lo, hi);
        }
        v[r] = a;
    }
    __syncthreads();
    int flip = 0;
    if (mode == 2) {
        line.template run<1>(v, j, buf0 + l * ls, buf1 + l * ls, 1, tw, flip);
        const bool next = P.method != 1 && it + 1 < P.max_iter && !ran_out(P, it + 1);
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int x = j + r * L::TPL;
            v[r] = make_float2(__fmul_rn(v[r].x, P.scale), __fmul_rn(v[r].y, P.scale));
            if (valid && x < n) {
                P.data[base + x] = v[r];
                if (next)
                    v[r] = constrain(P, v[r], P.flags[base + x], 0.f, 0.f, 0.f, 0.f);
            }
        }
        if (!next)
            return;  // uniform over the CTA
        __syncthreads();
    }
    line.template run<-1>(v, j, buf0 + l * ls, buf1 + l * ls, 1, tw, flip);
    if (!valid)
        return;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int x = j + r * L::TPL;
        if (x < n)
            P.buf[base + x] = v[r];
    }
}

// ---- axes 1 and 0 (strided lines, KX adjacent lines per CTA) --------------
// mode 0: forward (axis 1) ; mode 1: inverse (axis 1)
// mode 2: axis 0 forward -> orig (the original spectrum) + core sum
// mode 3: axis 0 forward -> frequency-domain step -> inverse (iteration)
template <class L, int KX>
__global__ void __launch_bounds__(KX *L::TPL) k_apple_s(AP P, L line, int axis, int mode, int it)
{
    if (mode != 2 && ran_out(P, it))
        return;
    extern __shared__ float2 smem[];
    __shared__ double red[32];
    const int n = line.size();
    const int ls = xslots<true>(n);
    float2 *buf0 = smem, *buf1 = smem + KX * ls, *tw = smem + 2 * KX * ls;
    copy_twiddles<L>(tw, axis == 0 ? P.tw0 : P.tw1, n);
    const long long inner = axis == 0 ? (long long)P.n1 * P.n2 : P.n2;
    const long long stride = inner;
    const long long ostride = (long long)P.n1 * P.n2;
    const unsigned gpo = (unsigned)((inner + KX - 1) / KX);
    const long long o = blockIdx.x / gpo;
    const long long q0 = (long long)(blockIdx.x - (unsigned)o * gpo) * KX;
    const int c = threadIdx.x % KX, j = threadIdx.x / KX;
    const long long q = q0 + c;
    const bool colok = q < inner;
    const long long base = (axis == 0 ? 0 : o * ostride) + (colok ? q : 0);
    float2 v[L::SLOTS];
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int k = j + r * L::TPL;
        v[r] = (colok && k < n) ? P.buf[base + k * stride] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    int flip = 0;
    if (mode == 1)
        line.template run<1, true>(v, j, buf0 + c, buf1 + c, KX, tw, flip);
    else
        line.template run<-1, true>(v, j, buf0 + c, buf1 + c, KX, tw, flip);
    double part = 0.0;
    if (mode >= 2) {
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int k = j + r * L::TPL;
            if (!(colok && k < n))
                continue;
            const long long vox = base + k * stride;
            const uint8_t fl = P.flags[vox];
            float2 ft = v[r];
            if (mode == 2) {
                P.orig[vox] = ft;
            } else {
                if (P.evlp && hypotf(ft.x, ft.y) > P.evlp[vox])
                    ft = make_float2(__fmul_rn(ft.x, P.ee), __fmul_rn(ft.y, P.ee));
                if (!(fl & F_CORE)) {
                    float2 og = P.orig[vox];
                    if (P.method == 1 && vox == 0) {  // (orig + ft) / 2 at the DC term
                        og = make_float2(__fmul_rn(__fadd_rn(og.x, ft.x), 0.5f),
                                         __fmul_rn(__fadd_rn(og.y, ft.y), 0.5f));
                        P.orig[0] = og;
                    }
                    ft = og;
                }
            }
            if (fl & F_CORE)
                part += (double)hypotf(ft.x, ft.y);
            v[r] = ft;
        }
        // block sum of the core magnitudes
        for (int s = 16; s > 0; s >>= 1)
            part += __shfl_xor_sync(0xffffffffu, part, s);
        if ((threadIdx.x & 31) == 0)
            red[threadIdx.x >> 5] = part;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
                t += red[w];
            atomicAdd(P.state + (mode == 2 ? 0 : it + 1), t);
        }
        if (mode == 2)
            return;
        __syncthreads();
        line.template run<1, true>(v, j, buf0 + c, buf1 + c, KX, tw, flip);
    }
    if (!colok)
        return;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int k = j + r * L::TPL;
        if (k < n)
            P.buf[base + k * stride] = v[r];
    }
}

// init_state (it < 0) or the stopping test of iteration `it`, in float32 as
// the reference's NumPy scalars: state = sum / N, diff = state - prev,
// norm = diff at iteration 0, stop when |diff / norm| < min_diff.
__global__ void k_apple_dec(AP P, int it)
{
    AppleCtl *c = P.ctl;
    if (it < 0) {
        c->prev = __fdiv_rn((float)P.state[0], (float)P.N);
        return;
    }
    if (c->stop != 0 && c->stop <= it)
        return;
    const float cur = __fdiv_rn((float)P.state[it + 1], (float)P.N);
    const float diff = __fsub_rn(cur, c->prev);
    c->iters = it + 1;
    if (it == 0) {
        c->norm = diff;
    } else if (fabsf(__fdiv_rn(diff, c->norm)) < P.min_diff) {
        c->stop = it + 1;
        return;
    }
    c->prev = cur;
}

// data = f.real + 0i (the state before the loop)
__global__ void k_apple_load(AP P)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < P.N;
         v += (long long)gridDim.x * blockDim.x)
        P.data[v] = make_float2(P.freal[v], 0.f);
}

// ---- voxel flags (FP64, the reference's formulas and operation order) ----
// The per-voxel formulas separate: per axis the fftfreq value, its square,
// k = 2 pi f and the ellipsoid terms ((i - c) / (c - shell))^2; per (i0, i2)
// sqrt(max(2 km kxz - kxz^2, 0)) with kxz = 2 pi sqrt(fx^2 + fz^2).  Every
// value is the one NumPy computes (same operations, same order), so the
// flags match the reference bit for bit.
struct FlagTables {
    double *sq[3];     // f^2 per axis
    double *ky;        // 2 pi f, axis 1
    double *eo[3];     // outer ellipsoid term per axis (shell 0)
    double *ei[3];     // inner ellipsoid term per axis (shell width)
    double *sroot;     // [n0 * n2]
};

__device__ __forceinline__ double fftfreq(int k, int n)
{
    // numpy.fft.fftfreq: integer frequency times 1.0 / n
    const int kk = k < (n - 1) / 2 + 1 ? k : k - n;
    return __dmul_rn((double)kk, __ddiv_rn(1.0, (double)n));
}

__device__ __forceinline__ double ell_term(int i, int n, double shell)
{
    const double c = n / 2.0;
    const double a = __ddiv_rn(__dsub_rn((double)i, c), __dsub_rn(c, shell));
    return __dmul_rn(a, a);
}

__global__ void k_apple_tables(int n0, int n1, int n2, double km, double shell_width, FlagTables T)
{
    const double twopi = 6.283185307179586;
    const int n[3] = {n0, n1, n2};
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int ax = 0; ax < 3; ++ax)
        if (t < n[ax]) {
            const double f = fftfreq(t, n[ax]);
            T.sq[ax][t] = __dmul_rn(f, f);
            if (ax == 1)
                T.ky[t] = __dmul_rn(twopi, f);
            T.eo[ax][t] = ell_term(t, n[ax], 0.0);
            T.ei[ax][t] = ell_term(t, n[ax], shell_width);
        }
    for (long long q = t; q < (long long)n0 * n2; q += (long long)gridDim.x * blockDim.x) {
        const int i0 = (int)(q / n2), i2 = (int)(q % n2);
        const double fx = fftfreq(i0, n0), fz = fftfreq(i2, n2);
        const double kxz = __dmul_rn(twopi, sqrt(__dadd_rn(__dmul_rn(fx, fx), __dmul_rn(fz, fz))));
        double root = __dsub_rn(__dmul_rn(__dmul_rn(2.0, km), kxz), __dmul_rn(kxz, kxz));
        if (root < 0.0)
            root = 0.0;
        T.sroot[q] = sqrt(root);
    }
}

__global__ void k_apple_flags(int n0, int n1, int n2, double km, int use_shell, FlagTables T, const uint8_t *mask,
                              const uint8_t *shell, uint8_t *flags)
{
    // grid (ceil(n2/32), ceil(n1/8), n0), blocks of 32 x 8
    const double twopi = 6.283185307179586;
    const double sqrt2km = __dmul_rn(1.4142135623730951, km);
    {
        const int i2 = (int)(blockIdx.x * 32 + threadIdx.x), i1 = (int)(blockIdx.y * 8 + threadIdx.y);
        const int i0 = (int)blockIdx.z;
        if (i2 >= n2 || i1 >= n1)
            return;
        const long long v = ((long long)i0 * n1 + i1) * n2 + i2;
        bool core = fabs(T.ky[i1]) > T.sroot[(long long)i0 * n2 + i2];
        const double kr = __dmul_rn(twopi, sqrt(__dadd_rn(__dadd_rn(T.sq[0][i0], T.sq[1][i1]), T.sq[2][i2])));
        if (kr > sqrt2km)
            core = false;
        uint8_t f = core ? F_CORE : 0;
        const bool outer = __dadd_rn(__dadd_rn(T.eo[0][i0], T.eo[1][i1]), T.eo[2][i2]) > 1.0;
        if (outer)
            f |= F_SPOV;
        if (use_shell && outer != (__dadd_rn(__dadd_rn(T.ei[0][i0], T.ei[1][i1]), T.ei[2][i2]) > 1.0))
            f |= F_SHELL;
        if (shell && shell[v])
            f |= F_SHELL;
        if (mask && mask[v])
            f |= F_MASK;
        flags[v] = f;
    }
}

// Tables in a scratch block of flag_table_bytes() bytes; then the flags.
// `shell` (device bytes, nonzero = background shell, or NULL) adds a shell
// given voxel by voxel to the computed one.
size_t flag_table_bytes(int n0, int n1, int n2)
{
    return (size_t)(3 * (n0 + n1 + n2) + n1 + (long long)n0 * n2 + 8) * 8;
}

cudaError_t compute_flags(int n0, int n1, int n2, double km, int use_shell, double shell_width, const uint8_t *mask,
                          const uint8_t *shell, uint8_t *flags, double *tab, cudaStream_t s)
{
    FlagTables T;
    double *p = tab;
    const int n[3] = {n0, n1, n2};
    for (int ax = 0; ax < 3; ++ax) {
        T.sq[ax] = p;
        p += n[ax];
        T.eo[ax] = p;
        p += n[ax];
        T.ei[ax] = p;
        p += n[ax];
    }
    T.ky = p;
    p += n1;
    T.sroot = p;
    const long long q = (long long)n0 * n2;
    const int mx = std::max(n0, std::max(n1, n2));
    const unsigned tg = (unsigned)std::max<long long>((mx + 255) / 256, std::min<long long>((q + 255) / 256, 1024));
    k_apple_tables<<<tg, 256, 0, s>>>(n0, n1, n2, km, shell_width, T);
    const dim3 fg((unsigned)((n2 + 31) / 32), (unsigned)((n1 + 7) / 8), (unsigned)n0), fb(32, 8);
    k_apple_flags<<<fg, fb, 0, s>>>(n0, n1, n2, km, use_shell, T, mask, shell, flags);
    return cudaGetLastError();
}

// ---- envelope --------------------------------------------------------------
struct EnvGeom {
    int n0, n1, n2, msh;
    int off0, off1, off2;  // where the volume sits in the padded cube
};

__device__ __forceinline__ int wrapi(int i, int n) { return ((i % n) + n) % n; }

__device__ __forceinline__ double magnitude(float2 o) { return (double)hypotf(o.x, o.y); }
__device__ __forceinline__ double magnitude(double2 o) { return hypot(o.x, o.y); }

// hull_pad = fftshift(|orig|, core -> NaN) inside the slice, 0 outside;
// cpad = fftshift(core) inside the slice.  C2 = float2 (complex64 spectrum,
// float32 hull) or double2 (complex128, float64 hull); the core is bit 0 of
// flags[v].
template <typename C2>
__global__ void k_env_pad(EnvGeom G, const C2 *orig, const uint8_t *flags, double *hp, uint8_t *cpad)
{
    // grid (ceil(msh/32), ceil(msh/8), msh), blocks of 32 x 8
    {
        const int c = (int)(blockIdx.x * 32 + threadIdx.x), b = (int)(blockIdx.y * 8 + threadIdx.y);
        const int a = (int)blockIdx.z;
        if (c >= G.msh || b >= G.msh)
            return;
        const long long p = ((long long)a * G.msh + b) * G.msh + c;
        const int i0 = a - G.off0, i1 = b - G.off1, i2 = c - G.off2;
        double h = 0.0;
        uint8_t cp = 0;
        if (i0 >= 0 && i0 < G.n0 && i1 >= 0 && i1 < G.n1 && i2 >= 0 && i2 < G.n2) {
            const int s0 = wrapi(i0 - G.n0 / 2, G.n0), s1 = wrapi(i1 - G.n1 / 2, G.n1),
                      s2 = wrapi(i2 - G.n2 / 2, G.n2);
            const long long v = ((long long)s0 * G.n1 + s1) * G.n2 + s2;
            if (flags[v] & F_CORE) {
                h = __longlong_as_double(0x7ff8000000000000ll);
                cp = 1;
            } else {
                h = magnitude(orig[v]);
            }
        }
        hp[p] = h;
        cpad[p] = cp;
    }
}

// out = core ? in transposed over the first two axes : in; counts NaNs left
__global__ void k_env_swap(EnvGeom G, const double *in, const uint8_t *cpad, double *out, unsigned int *nan_count)
{
    // grid (ceil(msh/32), ceil(msh/8), msh), blocks of 32 x 8; every lane
    // reaches the warp sum
    unsigned int cnt = 0;
    const int c = (int)(blockIdx.x * 32 + threadIdx.x), b = (int)(blockIdx.y * 8 + threadIdx.y);
    const int a = (int)blockIdx.z;
    if (c < G.msh && b < G.msh) {
        const long long p = ((long long)a * G.msh + b) * G.msh + c;
        double h = in[p];
        if (cpad[p])
            h = in[((long long)b * G.msh + a) * G.msh + c];
        out[p] = h;
        cnt = (h != h);
    }
    for (int s = 16; s > 0; s >>= 1)
        cnt += __shfl_xor_sync(0xffffffffu, cnt, s);
    if ((threadIdx.x & 31) == 0 && cnt)
        atomicAdd(nan_count, cnt);
}

// Exact Euclidean feature transform (Maurer, Qi, Raghavan, IEEE PAMI 25(2),
// 2003): per axis, the lower envelope of the sites' distance parabolas along
// every line; axes in order 0, 1, 2; a tie goes to the earlier site.
// ft holds the linear index of the nearest known voxel, -1 for none yet.
__global__ void k_edt_init(long long M, const double *hp, int *ft)
{
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < M;
         p += (long long)gridDim.x * blockDim.x)
        ft[p] = (hp[p] != hp[p]) ? -1 : (int)p;
}

__global__ void k_edt_pass(int msh, int d, int *ft, int *scratch)
{
    const long long nl = (long long)msh * msh;
    const long long line = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= nl)
        return;
    const long long m2 = (long long)msh * msh;
    // fixed coordinates of the line
    int co[3];
    const int u = (int)(line / msh), w = (int)(line % msh);
    if (d == 0) {
        co[1] = u;
        co[2] = w;
    } else if (d == 1) {
        co[0] = u;
        co[2] = w;
    } else {
        co[0] = u;
        co[1] = w;
    }
    const long long strides[3] = {m2, msh, 1};
    co[d] = 0;
    const long long base = (long long)co[0] * m2 + (long long)co[1] * msh + co[2];
    const long long st = strides[d];
    int *f = scratch + line * 2 * msh;  // copy of the line's features
    int *g = f + msh;                   // site stack (positions)
    auto coord = [&](int idx, int k) -> long long {
        return k == 0 ? idx / m2 : (k == 1 ? (idx / msh) % msh : idx % msh);
    };
    for (int i = 0; i < msh; ++i)
        f[i] = ft[base + i * st];
    int l = -1;
    for (int i = 0; i < msh; ++i) {
        const int fi = f[i];
        if (fi < 0)
            continue;
        long long wR = 0;
        for (int k = 0; k < 3; ++k)
            if (k != d) {
                const long long t = coord(fi, k) - co[k];
                wR += t * t;
            }
        const long long fd = coord(fi, d);
        while (l >= 1) {
            const int iu = f[g[l - 1]], iv = f[g[l]];
            const long long a = coord(iv, d) - coord(iu, d);
            const long long b = fd - coord(iv, d);
            const long long c = a + b;
            long long uR = 0, vR = 0;
            for (int k = 0; k < 3; ++k)
                if (k != d) {
                    const long long tu = coord(iu, k) - co[k], tv = coord(iv, k) - co[k];
                    uR += tu * tu;
                    vR += tv * tv;
                }
            if (c * vR - b * uR - a * wR - a * b * c <= 0)
                break;
            --l;
        }
        g[++l] = i;
    }
    if (l < 0)
        return;
    const int maxl = l;
    l = 0;
    auto dist = [&](int idx, int i) -> long long {
        long long s = 0;
        for (int k = 0; k < 3; ++k) {
            const long long t = coord(idx, k) - (k == d ? i : co[k]);
            s += t * t;
        }
        return s;
    };
    for (int i = 0; i < msh; ++i) {
        long long d1 = dist(f[g[l]], i);
        while (l < maxl) {
            const long long d2 = dist(f[g[l + 1]], i);
            if (d1 <= d2)
                break;
            d1 = d2;
            ++l;
        }
        ft[base + i * st] = f[g[l]];
    }
}

__global__ void k_edt_gather(long long M, const int *ft, const double *in, double *out)
{
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < M;
         p += (long long)gridDim.x * blockDim.x)
        out[p] = ft[p] >= 0 ? in[ft[p]] : in[p];
}

// scipy.ndimage.gaussian_filter (mode constant 0): per axis in order 0, 1,
// 2, acc = x[i] w0 + sum_{j = r..1} (x[i+j] + x[i-j]) w_j in FP64, rounded
// to the hull's type T (float32 or float64) after each axis.  Axis 0 reads the padded cube's slice (the
// fftshifted hull); the last axis writes ifftshift(result) (the envelope in
// FFT order).  A 32 x 8 block stages its inputs as doubles in shared memory
// (one conversion per input): for axes 0 and 1 the block covers 32 x2
// positions and 8 consecutive positions along the filtered axis, for axis 2
// 32 consecutive x2 positions (the filtered axis) and 8 x1 rows.
constexpr int GAUSS_RMAX = 64;  // radius limit (sigma <= 15.9, volumes <= 1590)

template <typename T>
__global__ void __launch_bounds__(256) k_env_gauss(EnvGeom G, int axis, const double *hp, const T *in, T *out,
                                                   const double *w, int r)
{
    extern __shared__ double gx[];  // the staged inputs with halo
    const int n[3] = {G.n0, G.n1, G.n2};
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    int ii[3];
    auto input = [&](int a0, int a1, int a2) -> double {
        if (a0 < 0 || a0 >= G.n0 || a1 < 0 || a1 >= G.n1 || a2 < 0 || a2 >= G.n2)
            return 0.0;
        if (axis == 0)
            return (double)(T)hp[((long long)(a0 + G.off0) * G.msh + (a1 + G.off1)) * G.msh + (a2 + G.off2)];
        return (double)in[((long long)a0 * G.n1 + a1) * G.n2 + a2];
    };
    double acc;
    if (axis < 2) {
        // grid (ceil(n2/32), ceil(n_axis/8), n_other); smem [(8 + 2r)][32]
        const int a2 = (int)blockIdx.x * 32 + tx;
        const int s0 = (int)blockIdx.y * 8 - r;  // first staged position along the axis
        const int other = (int)blockIdx.z;
        const int rows = 8 + 2 * r;
        for (int t = tid; t < rows * 32; t += 256) {
            const int k = s0 + t / 32, c = (int)blockIdx.x * 32 + (t & 31);
            gx[t] = axis == 0 ? input(k, other, c) : input(other, k, c);
        }
        __syncthreads();
        const int k = (int)blockIdx.y * 8 + ty;
        if (k >= n[axis] || a2 >= G.n2)
            return;
        ii[axis] = k;
        ii[axis == 0 ? 1 : 0] = other;
        ii[2] = a2;
        const double *col = gx + (ty + r) * 32 + tx;
        acc = __dmul_rn(col[0], w[r]);
        for (int j = r; j >= 1; --j)
            acc = __dadd_rn(acc, __dmul_rn(__dadd_rn(col[j * 32], col[-j * 32]), w[r + j]));
    } else {
        // grid (ceil(n2/32), ceil(n1/8), n0); smem [8][32 + 2r]
        const int wdt = 32 + 2 * r;
        const int s2 = (int)blockIdx.x * 32 - r;
        for (int t = tid; t < 8 * wdt; t += 256) {
            const int row = t / wdt, c = t - row * wdt;
            gx[t] = input((int)blockIdx.z, (int)blockIdx.y * 8 + row, s2 + c);
        }
        __syncthreads();
        const int a1 = (int)blockIdx.y * 8 + ty, a2 = (int)blockIdx.x * 32 + tx;
        if (a1 >= G.n1 || a2 >= G.n2)
            return;
        ii[0] = (int)blockIdx.z;
        ii[1] = a1;
        ii[2] = a2;
        const double *row = gx + ty * wdt + tx + r;
        acc = __dmul_rn(row[0], w[r]);
        for (int j = r; j >= 1; --j)
            acc = __dadd_rn(acc, __dmul_rn(__dadd_rn(row[j], row[-j]), w[r + j]));
    }
    long long o = ((long long)ii[0] * G.n1 + ii[1]) * G.n2 + ii[2];
    if (axis == 2) {  // ifftshift: out[k] = g[(k + n/2) mod n]  =>  g[i] -> out[i - n/2]
        const int s0 = wrapi(ii[0] - G.n0 / 2, G.n0), s1 = wrapi(ii[1] - G.n1 / 2, G.n1),
                  s2 = wrapi(ii[2] - G.n2 / 2, G.n2);
        o = ((long long)s0 * G.n1 + s1) * G.n2 + s2;
    }
    out[o] = (T)acc;
}

// envelope_gauss (apple.py:289-350) of the spectrum `orig` (n0 == n2; C2 =
// float2 for complex64, double2 for complex128) with the core in bit 0 of
// flags, written to `out` (type T of the hull: float or double) in FFT
// order.  Scratch: hp0, hp1 (msh^3 doubles, msh = max(n0, n1)), cpad (msh^3
// bytes), ft (msh^3 ints), scratch (2 msh^3 ints), g0, g1 (n0 n1 n2 values
// of T), the Gaussian's 2 gr + 1 weights on the device and a NaN counter
// that is 0.  Synchronous: the NaN count decides whether the feature
// transform runs.
struct EnvWork {
    double *hp0, *hp1;
    uint8_t *cpad;
    int *ft, *scratch;
    void *g0, *g1;
    const double *gw;
    unsigned int *nan_count;
};

template <typename C2, typename T>
cudaError_t run_envelope(int n0, int n1, int n2, int gr, const C2 *orig, const uint8_t *flags, T *out,
                         const EnvWork &W, cudaStream_t s)
{
    cudaError_t e;
    EnvGeom G{};
    G.n0 = n0;
    G.n1 = n1;
    G.n2 = n2;
    G.msh = std::max(n0, n1);
    const int dsh = std::abs(n1 - n0) / 2;
    if (n0 > n1) {
        G.off0 = 0;
        G.off1 = dsh;
        G.off2 = 0;
    } else {
        G.off0 = dsh;
        G.off1 = 0;
        G.off2 = dsh;
    }
    const long long M = (long long)G.msh * G.msh * G.msh;
    const unsigned mg = (unsigned)std::min<long long>((M + 255) / 256, 152ll * 16);
    const dim3 cg((unsigned)((G.msh + 31) / 32), (unsigned)((G.msh + 7) / 8), (unsigned)G.msh), cb(32, 8);
    k_env_pad<C2><<<cg, cb, 0, s>>>(G, orig, flags, W.hp0, W.cpad);
    k_env_swap<<<cg, cb, 0, s>>>(G, W.hp0, W.cpad, W.hp1, W.nan_count);
    unsigned int nans = 0;
    if ((e = cudaMemcpyAsync(&nans, W.nan_count, 4, cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s)))
        return e;
    const double *hp = W.hp1;
    if (nans) {
        k_edt_init<<<mg, 256, 0, s>>>(M, W.hp1, W.ft);
        const long long nl = (long long)G.msh * G.msh;
        for (int ax = 0; ax < 3; ++ax)
            k_edt_pass<<<(unsigned)((nl + 127) / 128), 128, 0, s>>>(G.msh, ax, W.ft, W.scratch);
        k_edt_gather<<<mg, 256, 0, s>>>(M, W.ft, W.hp1, W.hp0);
        hp = W.hp0;
    }
    T *g0 = (T *)W.g0, *g1 = (T *)W.g1;
    const dim3 vb(32, 8);
    const dim3 g0g((unsigned)((n2 + 31) / 32), (unsigned)((n0 + 7) / 8), (unsigned)n1);
    const dim3 g1g((unsigned)((n2 + 31) / 32), (unsigned)((n1 + 7) / 8), (unsigned)n0);
    const size_t sm01 = (size_t)(8 + 2 * gr) * 32 * 8, sm2 = (size_t)8 * (32 + 2 * gr) * 8;
    const size_t smx = std::max(sm01, sm2);
    if (smx > 48 * 1024 &&
        (e = cudaFuncSetAttribute(k_env_gauss<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx)))
        return e;
    k_env_gauss<T><<<g0g, vb, sm01, s>>>(G, 0, hp, nullptr, g0, W.gw, gr);
    k_env_gauss<T><<<g1g, vb, sm01, s>>>(G, 1, hp, g0, g1, W.gw, gr);
    k_env_gauss<T><<<g1g, vb, sm2, s>>>(G, 2, hp, g1, out, W.gw, gr);
    return cudaGetLastError();
}

// ---- method "sh": min / max over the spillover (and shell) voxels and the
// histogram of all values in [fmin, fmax], for float32 or float64 data ------
// Order-preserving keys of the values (min / max by integer atomics).
template <typename T>
struct OrdKey;
template <>
struct OrdKey<float> {
    __device__ static unsigned long long of(float f)
    {
        const unsigned int b = __float_as_uint(f);
        return (b >> 31) ? (unsigned long long)(~b) : (unsigned long long)(b | 0x80000000u);
    }
    __host__ __device__ static float val(unsigned long long k)
    {
        const unsigned int u = (unsigned int)k;
        const unsigned int b = (u >> 31) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
        return __uint_as_float(b);
#else
        float f;
        memcpy(&f, &b, 4);
        return f;
#endif
    }
};
template <>
struct OrdKey<double> {
    __device__ static unsigned long long of(double f)
    {
        const unsigned long long b = (unsigned long long)__double_as_longlong(f);
        return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
    }
    __host__ __device__ static double val(unsigned long long k)
    {
        const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
#ifdef __CUDA_ARCH__
        return __longlong_as_double((long long)b);
#else
        double f;
        memcpy(&f, &b, 8);
        return f;
#endif
    }
};

__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }

// One spatial constraint's arguments: the real parts at data[v * stride]
// (stride 2 for complex data), the voxel flags, and the "sh" state.
template <typename T>
struct ConsArgs {
    T *data;
    long long N;
    int stride;
    const uint8_t *flags;
    int method;  // 0 nn, 1 sh
    int has_mask;
    unsigned long long *keys;  // [2] min, max keys (method "sh")
    unsigned int *hist;        // [HIST_BINS]
    const T *edges;            // [HIST_BINS + 1]
    const T *th;               // lo, hi, fmin, fmax
    const int *stop;           // with `it`: skip iterations after the stop (NULL: never)
    int it;
};

template <typename T>
__device__ __forceinline__ bool cons_skip(const ConsArgs<T> &C)
{
    if (!C.stop)
        return false;
    const int s = *(volatile const int *)C.stop;
    return s != 0 && s <= C.it;
}

template <typename T>
__global__ void k_sh_minmax(ConsArgs<T> C)
{
    if (cons_skip(C))
        return;
    unsigned long long mn = ~0ull, mx = 0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < C.N;
         v += (long long)gridDim.x * blockDim.x) {
        if (C.flags[v] & (F_SPOV | F_SHELL)) {
            const unsigned long long k = OrdKey<T>::of(C.data[v * C.stride]);
            mn = min(mn, k);
            mx = max(mx, k);
        }
    }
    for (int s = 16; s > 0; s >>= 1) {
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, s));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, s));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&C.keys[0], mn);
        atomicMax(&C.keys[1], mx);
    }
}

// numpy.histogram's bin of x for equal bins (arithmetic in the data's type):
// index = int(((x - first) / (last - first)) * bins), the last edge in the
// last bin, then one-step corrections against the edges.
template <typename T>
__global__ void k_sh_hist(ConsArgs<T> C)
{
    if (cons_skip(C))
        return;
    __shared__ unsigned int h[HIST_BINS];
    for (int i = threadIdx.x; i < HIST_BINS; i += blockDim.x)
        h[i] = 0;
    __syncthreads();
    const T first = C.edges[0], last = C.edges[HIST_BINS];
    const T denom = rn_sub(last, first);
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < C.N;
         v += (long long)gridDim.x * blockDim.x) {
        const T x = C.data[v * C.stride];
        if (!(x >= first && x <= last))
            continue;
        int idx = (int)rn_mul(rn_div(rn_sub(x, first), denom), (T)HIST_BINS);
        idx = min(max(idx, 0), HIST_BINS);  // (a zero-width range gives no NaN index)
        if (idx == HIST_BINS)
            idx -= 1;
        if (idx > 0 && x < C.edges[idx])
            idx -= 1;
        if (x >= C.edges[idx + 1] && idx != HIST_BINS - 1)
            idx += 1;
        idx = min(max(idx, 0), HIST_BINS - 1);
        atomicAdd(&h[idx], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < HIST_BINS; i += blockDim.x)
        if (h[i])
            atomicAdd(&C.hist[i], h[i]);
}

// The constraint applied in place (constraint_nn / constraint_sh called on
// their own): the real part constrained, the imaginary part zeroed.
template <typename T>
__global__ void k_constrain(ConsArgs<T> C)
{
    T lo = T(0), hi = T(0), fmin = T(0), fmax = T(0);
    if (C.method == 1) {
        lo = C.th[0];
        hi = C.th[1];
        fmin = C.th[2];
        fmax = C.th[3];
    }
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < C.N;
         v += (long long)gridDim.x * blockDim.x) {
        T *p = C.data + v * C.stride;
        p[0] = constrain_re<T>(C.method, C.has_mask, p[0], C.flags[v], fmin, fmax, lo, hi);
        if (C.stride == 2)
            p[1] = T(0);
    }
}

// numpy.linspace(first, last, 101) in the data's type (numpy.histogram's
// edges; first == last widened by 0.5 each way first), as numpy evaluates
// it: k * step + first, the last edge set to `last`.
template <typename T>
void hist_edges(T fmin, T fmax, T *edges)
{
    T first = fmin, last = fmax;
    if (first == last) {
        first = first - T(0.5);
        last = last + T(0.5);
    }
    const T delta = last - first;
    const T step = delta / (T)HIST_BINS;
    for (int k = 0; k <= HIST_BINS; ++k) {
        volatile T y = (T)k * step;  // no contraction into a fused multiply-add
        edges[k] = y + first;
    }
    edges[HIST_BINS] = last;
}

// count_to_half of apple.py:266-278 on counts a[0..len)
int count_to_half(const unsigned int *a, int len, int step)
{
    int num = 0;
    for (int i = 1; i < len; ++i) {
        if ((double)a[i * step] < (double)a[0] / 2.0)
            break;
        ++num;
    }
    return num;
}

// constraint_sh's thresholds from the 100 counts (apple.py:91-103): the
// histogram's peak, the bins down to half its count either side, the bin
// centres edge[k + 1] - de / 2; th = lo, hi, fmin, fmax.
template <typename T>
void sh_thresholds(const unsigned int *hist, const T *edges, T fmin, T fmax, T *th)
{
    int idx_c = 0;
    for (int k = 1; k < HIST_BINS; ++k)
        if (hist[k] > hist[idx_c])
            idx_c = k;
    const int idx_start = idx_c - (idx_c > 0 ? count_to_half(hist + idx_c - 1, idx_c, -1) : 0);
    const int idx_end = idx_c + count_to_half(hist + idx_c, HIST_BINS - idx_c, 1);
    const T de = edges[1] - edges[0];
    const T half = de / T(2);
    th[0] = edges[idx_start + 1] - half;
    th[1] = edges[idx_end + 1] - half;
    th[2] = fmin;
    th[3] = fmax;
}

// The "sh" thresholds of the values C.data (synchronous: the min / max keys
// and the counts come to the host).  C.keys, C.hist and C.edges point into
// the device workspace; the thresholds are copied to C.th.  *stopped is set
// when the iteration `C.it` lies after the loop's stop (nothing computed).
template <typename T>
cudaError_t sh_prepare(ConsArgs<T> C, unsigned eg, cudaStream_t s, bool *stopped)
{
    cudaError_t e;
    const unsigned long long k0[2] = {~0ull, 0ull};
    *stopped = false;
    if ((e = cudaMemcpyAsync(C.keys, k0, 16, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemsetAsync(C.hist, 0, HIST_BINS * 4, s)))
        return e;
    k_sh_minmax<T><<<eg, 256, 0, s>>>(C);
    unsigned long long keys[2];
    int stop = 0;
    if ((e = cudaMemcpyAsync(keys, C.keys, 16, cudaMemcpyDeviceToHost, s)))
        return e;
    if (C.stop && (e = cudaMemcpyAsync(&stop, C.stop, 4, cudaMemcpyDeviceToHost, s)))
        return e;
    if ((e = cudaStreamSynchronize(s)))
        return e;
    if (stop != 0 && stop <= C.it) {
        *stopped = true;
        return cudaSuccess;
    }
    const T fmin = OrdKey<T>::val(keys[0]), fmax = OrdKey<T>::val(keys[1]);
    T edges[HIST_BINS + 1];
    hist_edges<T>(fmin, fmax, edges);
    if ((e = cudaMemcpyAsync((void *)C.edges, edges, sizeof(edges), cudaMemcpyHostToDevice, s)))
        return e;
    k_sh_hist<T><<<eg, 256, 0, s>>>(C);
    unsigned int hist[HIST_BINS];
    if ((e = cudaMemcpyAsync(hist, C.hist, sizeof(hist), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
        return e;
    T th[4];
    sh_thresholds<T>(hist, edges, fmin, fmax, th);
    if ((e = cudaMemcpyAsync((void *)C.th, th, sizeof(th), cudaMemcpyHostToDevice, s)))
        return e;
    // the host arrays live until the copy ran
    return cudaStreamSynchronize(s);
}

// ---------------------------------------------------------------------------
template <class L>
size_t smem_x(int n)
{
    return (size_t)(2 * Cfg<L>::LPC * xslots<false>(n) + tw_slots(n)) * sizeof(float2);
}
template <class L>
size_t smem_s(int n)
{
    return (size_t)(2 * Cfg<L>::KX * xslots<true>(n) + tw_slots(n)) * sizeof(float2);
}

cudaError_t launch_x(const AP &P, int mode, int it, cudaStream_t s)
{
    return with_line(P.n2, [&](auto line) {
        using L = decltype(line);
        constexpr int LPC = Cfg<L>::LPC;
        const size_t sm = smem_x<L>(P.n2);
        cudaFuncSetAttribute(k_apple_x<L, LPC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        const long long lines = (long long)P.n0 * P.n1;
        k_apple_x<L, LPC><<<(unsigned)((lines + LPC - 1) / LPC), LPC * L::TPL, sm, s>>>(P, line, mode, it);
        return cudaGetLastError();
    });
}

cudaError_t launch_s(const AP &P, int axis, int mode, int it, cudaStream_t s)
{
    const int n = axis == 0 ? P.n0 : P.n1;
    return with_line(n, [&](auto line) {
        using L = decltype(line);
        constexpr int KX = Cfg<L>::KX;
        const size_t sm = smem_s<L>(n);
        cudaFuncSetAttribute(k_apple_s<L, KX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        const long long inner = axis == 0 ? (long long)P.n1 * P.n2 : P.n2;
        const long long outer = axis == 0 ? 1 : P.n0;
        const long long grid = outer * ((inner + KX - 1) / KX);
        k_apple_s<L, KX><<<(unsigned)grid, KX * L::TPL, sm, s>>>(P, line, axis, mode, it);
        return cudaGetLastError();
    });
}

struct Layout {
    size_t ctl, state, hist, edges, tw0, tw1, tw2, gw, ftab, flags, buf, orig, evlp, hp0, hp1, cpad, ft, scratch, g0,
        g1, total;
};

Layout layout_of(const odt_apple_desc &d)
{
    const long long N = (long long)d.n0 * d.n1 * d.n2;
    const long long msh = std::max(d.n0, d.n1);
    const long long M = msh * msh * msh;
    Layout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += (bytes + 255) / 256 * 256;
        return at;
    };
    L.ctl = take(sizeof(AppleCtl));
    L.state = take((size_t)(std::max(d.max_iter, 0) + 1) * 8);
    L.hist = take(HIST_BINS * 4);
    L.edges = take((HIST_BINS + 1) * 4);
    L.tw0 = take((size_t)d.n0 * 8);
    L.tw1 = take((size_t)d.n1 * 8);
    L.tw2 = take((size_t)d.n2 * 8);
    L.gw = take((size_t)(2 * std::max(d.gauss_radius, 0) + 1) * 8);
    L.ftab = take(flag_table_bytes(d.n0, d.n1, d.n2));
    L.flags = take((size_t)N);
    L.buf = take((size_t)N * 8);
    L.orig = take((size_t)N * 8);
    if (d.enforce_envelope != 0.0) {
        L.evlp = take((size_t)N * 4);
        L.hp0 = take((size_t)M * 8);
        L.hp1 = take((size_t)M * 8);
        L.cpad = take((size_t)M);
        L.ft = take((size_t)M * 4);
        L.scratch = take((size_t)msh * msh * 2 * msh * 4);
        L.g0 = take((size_t)N * 4);
        L.g1 = take((size_t)N * 4);
    }
    L.total = o;
    return L;
}

odt_status check_desc(const odt_apple_desc *d)
{
    if (!d)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL descriptor");
    if (d->n0 < 1 || d->n1 < 1 || d->n2 < 1)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "volume sizes must be positive");
    if (d->n0 != d->n2)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "`shape[0]` and `shape[2]` must be identical!");
    for (int n : {d->n0, d->n1, d->n2})
        if (!(n <= GenericLine::TPL * GenericLine::SLOTS || (n <= 4096 && (n & (n - 1)) == 0)))
            return (odt_status)set_error(ODT_ERR_UNSUPPORTED,
                                         "volume axes longer than 1024 must be powers of two up to 4096");
    if (!(d->enforce_envelope >= 0.0 && d->enforce_envelope <= 1.0))
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "`enforce_envelope` must be in interval [0, 1]");
    if (d->method != ODT_APPLE_NN && d->method != ODT_APPLE_SH && d->method != ODT_APPLE_NONE)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "unknown constraint method");
    if (d->max_iter < 0)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "max_iter must not be negative");
    if (d->enforce_envelope != 0.0 && (d->gauss_radius < 0 || !d->gauss_weights))
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "envelope needs the Gaussian weights");
    if (d->enforce_envelope != 0.0 && d->gauss_radius > GAUSS_RMAX)
        return (odt_status)set_error(ODT_ERR_UNSUPPORTED, "envelope Gaussian radius above 64 (volume axes above 1590)");
    if ((long long)d->n0 * d->n1 * d->n2 >= (1ll << 31))
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "volume too large (2^31 voxels or more)");
    return ODT_OK;
}

odt_status cuda_fail(const char *what, cudaError_t e)
{
    return (odt_status)set_error(ODT_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
}

std::vector<float2> twiddles(int n)
{
    std::vector<float2> t(n);
    for (int m = 0; m < n; ++m)
        t[m] = make_float2((float)std::cos(-2.0 * M_PI * m / n), (float)std::sin(-2.0 * M_PI * m / n));
    return t;
}

// ---- constraint_nn / constraint_sh / envelope_gauss called on their own --
odt_status check_helper(const odt_apple_desc *d, int32_t real_bits)
{
    if (!d)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL descriptor");
    if (d->n0 < 1 || d->n1 < 1 || d->n2 < 1)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "volume sizes must be positive");
    if ((long long)d->n0 * d->n1 * d->n2 >= (1ll << 31))
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "volume too large (2^31 voxels or more)");
    if (real_bits != 32 && real_bits != 64)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "real_bits must be 32 or 64");
    return ODT_OK;
}

odt_status check_envelope(const odt_apple_desc *d)
{
    if (d->n0 != d->n2)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "`shape[0]` and `shape[2]` must be identical!");
    if (d->gauss_radius < 0 || !d->gauss_weights)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "envelope needs the Gaussian weights");
    if (d->gauss_radius > GAUSS_RMAX)
        return (odt_status)set_error(ODT_ERR_UNSUPPORTED, "envelope Gaussian radius above 64 (volume axes above 1590)");
    const long long msh = std::max(d->n0, d->n1);
    if (msh * msh * msh >= (1ll << 31))
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "volume too large (max(n0, n1)^3 of 2^31 or more)");
    return ODT_OK;
}

struct HelperLayout {
    size_t ctl, hist, edges, ftab, flags, gw, hp0, hp1, cpad, ft, scratch, g0, g1, total;
};

// envelope == false: the constraint's workspace; true: the envelope's
HelperLayout helper_layout(const odt_apple_desc &d, bool envelope)
{
    const long long N = (long long)d.n0 * d.n1 * d.n2;
    HelperLayout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += (bytes + 255) / 256 * 256;
        return at;
    };
    L.ctl = take(64);  // min / max keys, thresholds (or the NaN counter)
    if (!envelope) {
        L.hist = take(HIST_BINS * 4);
        L.edges = take((HIST_BINS + 1) * 8);
        L.ftab = take(flag_table_bytes(d.n0, d.n1, d.n2));
        L.flags = take((size_t)N);
    } else {
        const long long msh = std::max(d.n0, d.n1);
        const long long M = msh * msh * msh;
        L.gw = take((size_t)(2 * std::max(d.gauss_radius, 0) + 1) * 8);
        L.hp0 = take((size_t)M * 8);
        L.hp1 = take((size_t)M * 8);
        L.cpad = take((size_t)M);
        L.ft = take((size_t)M * 4);
        L.scratch = take((size_t)msh * msh * 2 * msh * 4);
        L.g0 = take((size_t)N * 8);
        L.g1 = take((size_t)N * 8);
    }
    L.total = o;
    return L;
}

template <typename T>
cudaError_t constrain_impl(const odt_apple_desc &d, int is_complex, T *data, const uint8_t *mask,
                           const uint8_t *bg_shell, char *ws, const HelperLayout &L, cudaStream_t s)
{
    cudaError_t e;
    const long long N = (long long)d.n0 * d.n1 * d.n2;
    uint8_t *flags = (uint8_t *)(ws + L.flags);
    // spillover region (shell 0), the given shell and mask
    if ((e = compute_flags(d.n0, d.n1, d.n2, 1.0, 0, 0.0, mask, bg_shell, flags, (double *)(ws + L.ftab), s)))
        return e;
    ConsArgs<T> C{};
    C.data = data;
    C.N = N;
    C.stride = is_complex ? 2 : 1;
    C.flags = flags;
    C.method = d.method == ODT_APPLE_SH ? 1 : 0;
    C.has_mask = mask != nullptr;
    C.keys = (unsigned long long *)(ws + L.ctl);
    C.th = (const T *)(ws + L.ctl + 16);
    C.hist = (unsigned int *)(ws + L.hist);
    C.edges = (const T *)(ws + L.edges);
    const unsigned eg = (unsigned)std::min<long long>((N + 255) / 256, 152ll * 16);
    if (C.method == 1) {
        bool stopped;
        if ((e = sh_prepare<T>(C, eg, s, &stopped)))
            return e;
    }
    k_constrain<T><<<eg, 256, 0, s>>>(C);
    return cudaGetLastError();
}

template <typename C2, typename T>
cudaError_t envelope_impl(const odt_apple_desc &d, const C2 *ftdata, const uint8_t *core, T *out, char *ws,
                          const HelperLayout &L, cudaStream_t s)
{
    cudaError_t e;
    EnvWork W{};
    W.hp0 = (double *)(ws + L.hp0);
    W.hp1 = (double *)(ws + L.hp1);
    W.cpad = (uint8_t *)(ws + L.cpad);
    W.ft = (int *)(ws + L.ft);
    W.scratch = (int *)(ws + L.scratch);
    W.g0 = ws + L.g0;
    W.g1 = ws + L.g1;
    W.gw = (const double *)(ws + L.gw);
    W.nan_count = (unsigned int *)(ws + L.ctl);
    // (the weights are read on the host until run_envelope's first wait)
    if ((e = cudaMemcpyAsync(ws + L.gw, d.gauss_weights, (size_t)(2 * d.gauss_radius + 1) * 8,
                             cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemsetAsync(W.nan_count, 0, 4, s)))
        return e;
    return run_envelope<C2, T>(d.n0, d.n1, d.n2, d.gauss_radius, ftdata, core, out, W, s);
}

}  // namespace
}  // namespace odt

using namespace odt;

extern "C" {

odt_status odt_apple_workspace_size(const odt_apple_desc *desc, size_t *bytes)
{
    const odt_status st = check_desc(desc);
    if (st != ODT_OK)
        return st;
    if (!bytes)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL output pointer");
    *bytes = layout_of(*desc).total;
    return ODT_OK;
}

odt_status odt_apple_flags(const odt_apple_desc *desc, const uint8_t *mask, uint8_t *flags, void *workspace,
                           void *stream)
{
    const odt_status st = check_desc(desc);
    if (st != ODT_OK)
        return st;
    if (!flags || !workspace)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if ((uintptr_t)workspace % 256)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "misaligned pointer");
    const odt_apple_desc &d = *desc;
    const cudaError_t e = compute_flags(d.n0, d.n1, d.n2, (2.0 * M_PI * d.nm) / d.res, d.use_bg_shell,
                                        d.bg_shell_width, mask, nullptr, flags, (double *)workspace,
                                        (cudaStream_t)stream);
    return e == cudaSuccess ? ODT_OK : cuda_fail("apple flags", e);
}

odt_status odt_apple_flags_workspace_size(const odt_apple_desc *desc, size_t *bytes)
{
    const odt_status st = check_desc(desc);
    if (st != ODT_OK)
        return st;
    if (!bytes)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL output pointer");
    *bytes = flag_table_bytes(desc->n0, desc->n1, desc->n2);
    return ODT_OK;
}

odt_status odt_apple_correct(const odt_apple_desc *desc, const float *f_real, const uint8_t *mask, void *out,
                             void *workspace, size_t workspace_bytes, int32_t *iterations, void *stream)
{
    const odt_status st = check_desc(desc);
    if (st != ODT_OK)
        return st;
    if (!f_real || !out || !workspace)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL device pointer");
    const Layout L = layout_of(*desc);
    if (workspace_bytes < L.total)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "workspace too small");
    if ((uintptr_t)workspace % 256 || (uintptr_t)out % 8 || (uintptr_t)f_real % 4)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "misaligned pointer");
    const odt_apple_desc &d = *desc;
    cudaStream_t s = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    const long long N = (long long)d.n0 * d.n1 * d.n2;
    AP P{};
    P.n0 = d.n0;
    P.n1 = d.n1;
    P.n2 = d.n2;
    P.N = N;
    P.tw0 = (const float2 *)(ws + L.tw0);
    P.tw1 = (const float2 *)(ws + L.tw1);
    P.tw2 = (const float2 *)(ws + L.tw2);
    P.flags = (const uint8_t *)(ws + L.flags);
    P.evlp = d.enforce_envelope != 0.0 ? (const float *)(ws + L.evlp) : nullptr;
    P.ee = (float)d.enforce_envelope;
    P.orig = (float2 *)(ws + L.orig);
    P.buf = (float2 *)(ws + L.buf);
    P.data = (float2 *)out;
    P.freal = f_real;
    P.state = (double *)(ws + L.state);
    P.ctl = (AppleCtl *)(ws + L.ctl);
    P.method = d.method;
    P.max_iter = d.max_iter;
    P.min_diff = (float)d.min_diff;
    P.scale = 1.0f / (float)N;
    P.has_mask = mask != nullptr;
    P.hist = (unsigned int *)(ws + L.hist);
    P.edges = (const float *)(ws + L.edges);
    cudaError_t e;
    // tables
    {
        const std::vector<float2> t0 = twiddles(d.n0), t1 = twiddles(d.n1), t2 = twiddles(d.n2);
        if ((e = cudaMemcpyAsync(ws + L.tw0, t0.data(), t0.size() * 8, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(ws + L.tw1, t1.data(), t1.size() * 8, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(ws + L.tw2, t2.data(), t2.size() * 8, cudaMemcpyHostToDevice, s)))
            return cuda_fail("apple tables", e);
        if (P.evlp &&
            (e = cudaMemcpyAsync(ws + L.gw, d.gauss_weights, (size_t)(2 * d.gauss_radius + 1) * 8,
                                 cudaMemcpyHostToDevice, s)))
            return cuda_fail("apple tables", e);
        if ((e = cudaMemsetAsync(ws + L.ctl, 0, sizeof(AppleCtl), s)) ||
            (e = cudaMemsetAsync(ws + L.state, 0, (size_t)(std::max(d.max_iter, 0) + 1) * 8, s)))
            return cuda_fail("apple reset", e);
        // the tables must reach the device before the host vectors go
        if ((e = cudaStreamSynchronize(s)))
            return cuda_fail("apple tables", e);
    }
    const unsigned eg = (unsigned)std::min<long long>((N + 255) / 256, 152ll * 16);
    const double km = (2.0 * M_PI * d.nm) / d.res;
    if ((e = compute_flags(d.n0, d.n1, d.n2, km, d.use_bg_shell, d.bg_shell_width, mask, nullptr,
                           (uint8_t *)(ws + L.flags), (double *)(ws + L.ftab), s)))
        return cuda_fail("apple flags", e);
    // original spectrum: axis 2, 1 from f.real into buf, axis 0 into orig
    if ((e = launch_x(P, 0, -1, s)) || (e = launch_s(P, 1, 0, -1, s)) || (e = launch_s(P, 0, 2, -1, s)))
        return cuda_fail("apple spectrum", e);
    k_apple_dec<<<1, 1, 0, s>>>(P, -1);
    if (P.evlp) {
        EnvWork W{};
        W.hp0 = (double *)(ws + L.hp0);
        W.hp1 = (double *)(ws + L.hp1);
        W.cpad = (uint8_t *)(ws + L.cpad);
        W.ft = (int *)(ws + L.ft);
        W.scratch = (int *)(ws + L.scratch);
        W.g0 = ws + L.g0;
        W.g1 = ws + L.g1;
        W.gw = (const double *)(ws + L.gw);
        W.nan_count = &P.ctl->nan_count;
        if ((e = run_envelope<float2, float>(d.n0, d.n1, d.n2, d.gauss_radius, P.orig, P.flags,
                                             (float *)(ws + L.evlp), W, s)))
            return cuda_fail("apple envelope", e);
    }
    if (d.max_iter == 0 || d.method == ODT_APPLE_SH)
        k_apple_load<<<eg, 256, 0, s>>>(P);  // data = f.real
    int done = 0;
    AppleCtl host_ctl{};
    for (int it0 = 0; it0 < d.max_iter; it0 += CHUNK) {
        const int it1 = std::min(d.max_iter, it0 + CHUNK);
        for (int it = it0; it < it1; ++it) {
            if (d.method != ODT_APPLE_SH) {
                if (it == 0 && (e = launch_x(P, 1, 0, s)))
                    return cuda_fail("apple iteration", e);
            } else {
                // constraint_sh: min / max over the spillover region, the
                // histogram, and the thresholds (host, from 100 counts)
                ConsArgs<float> C{};
                C.data = (float *)P.data;
                C.N = N;
                C.stride = 2;
                C.flags = P.flags;
                C.method = 1;
                C.keys = &P.ctl->minkey;
                C.hist = P.hist;
                C.edges = P.edges;
                C.th = &P.ctl->lo;
                C.stop = &P.ctl->stop;
                C.it = it;
                bool stopped = false;
                if ((e = sh_prepare<float>(C, eg, s, &stopped)))
                    return cuda_fail("apple sh", e);
                if (stopped)
                    break;
                if ((e = launch_x(P, 3, it, s)))
                    return cuda_fail("apple iteration", e);
            }
            if ((e = launch_s(P, 1, 0, it, s)) || (e = launch_s(P, 0, 3, it, s)))
                return cuda_fail("apple iteration", e);
            k_apple_dec<<<1, 1, 0, s>>>(P, it);
            if ((e = launch_s(P, 1, 1, it, s)) || (e = launch_x(P, 2, it, s)))
                return cuda_fail("apple iteration", e);
        }
        if ((e = cudaMemcpyAsync(&host_ctl, P.ctl, sizeof(AppleCtl), cudaMemcpyDeviceToHost, s)) ||
            (e = cudaStreamSynchronize(s)))
            return cuda_fail("apple iteration", e);
        done = host_ctl.iters;
        if (host_ctl.stop != 0)
            break;
    }
    if ((e = cudaStreamSynchronize(s)))
        return cuda_fail("apple", e);
    if (iterations)
        *iterations = done;
    return ODT_OK;
}

odt_status odt_apple_constrain_workspace_size(const odt_apple_desc *desc, size_t *bytes)
{
    const odt_status st = check_helper(desc, 32);
    if (st != ODT_OK)
        return st;
    if (!bytes)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL output pointer");
    *bytes = helper_layout(*desc, false).total;
    return ODT_OK;
}

odt_status odt_apple_constrain(const odt_apple_desc *desc, int32_t real_bits, int32_t is_complex, void *data,
                               const uint8_t *mask, const uint8_t *bg_shell, void *workspace, size_t workspace_bytes,
                               void *stream)
{
    const odt_status st = check_helper(desc, real_bits);
    if (st != ODT_OK)
        return st;
    if (desc->method != ODT_APPLE_NN && desc->method != ODT_APPLE_SH)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "constraint method must be nn or sh");
    if (is_complex != 0 && is_complex != 1)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "is_complex must be 0 or 1");
    if (!data || !workspace)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL device pointer");
    const HelperLayout L = helper_layout(*desc, false);
    if (workspace_bytes < L.total)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "workspace too small");
    if ((uintptr_t)workspace % 256 || (uintptr_t)data % (real_bits / 8))
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "misaligned pointer");
    cudaStream_t s = (cudaStream_t)stream;
    const cudaError_t e =
        real_bits == 32
            ? constrain_impl<float>(*desc, is_complex, (float *)data, mask, bg_shell, (char *)workspace, L, s)
            : constrain_impl<double>(*desc, is_complex, (double *)data, mask, bg_shell, (char *)workspace, L, s);
    return e == cudaSuccess ? ODT_OK : cuda_fail("apple constraint", e);
}

odt_status odt_apple_envelope_workspace_size(const odt_apple_desc *desc, size_t *bytes)
{
    odt_status st = check_helper(desc, 32);
    if (st == ODT_OK)
        st = check_envelope(desc);
    if (st != ODT_OK)
        return st;
    if (!bytes)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL output pointer");
    *bytes = helper_layout(*desc, true).total;
    return ODT_OK;
}

odt_status odt_apple_envelope(const odt_apple_desc *desc, int32_t real_bits, const void *ftdata, const uint8_t *core,
                              void *envelope, void *workspace, size_t workspace_bytes, void *stream)
{
    odt_status st = check_helper(desc, real_bits);
    if (st == ODT_OK)
        st = check_envelope(desc);
    if (st != ODT_OK)
        return st;
    if (!ftdata || !core || !envelope || !workspace)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL device pointer");
    const HelperLayout L = helper_layout(*desc, true);
    if (workspace_bytes < L.total)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "workspace too small");
    const size_t rb = (size_t)real_bits / 8;
    if ((uintptr_t)workspace % 256 || (uintptr_t)ftdata % (2 * rb) || (uintptr_t)envelope % rb)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "misaligned pointer");
    cudaStream_t s = (cudaStream_t)stream;
    const cudaError_t e =
        real_bits == 32 ? envelope_impl<float2, float>(*desc, (const float2 *)ftdata, core, (float *)envelope,
                                                       (char *)workspace, L, s)
                        : envelope_impl<double2, double>(*desc, (const double2 *)ftdata, core, (double *)envelope,
                                                         (char *)workspace, L, s);
    return e == cudaSuccess ? ODT_OK : cuda_fail("apple envelope", e);
}

}  // extern "C"
