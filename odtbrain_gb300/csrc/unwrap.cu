// Sinogram preparation on the GPU: odtbrain.sinogram_as_rytov /
// sinogram_as_radon (odtbrain/_prepare_sino.py:60-182) and the helper
// align_unwrapped (odtbrain/_prepare_sino.py:7-46).
//
// Per call, in the precision T of the sinogram (float for complex64, double
// for complex128), all stream-ordered:
//   k_phase          phi = angle(u / u0), lna = log|u / u0| (rytov; the
//                    complex division is Smith's algorithm, as NumPy's) or
//                    phi = angle(u) (radon)
//   2D sinograms     k_unwrap_rows: numpy.unwrap along each detector line,
//                    sequential per line in NumPy's operation order
//   3D sinograms     per frame the reliability-sorted unwrapping of Herraez
//                    et al. (Appl. Opt. 41, 7437, 2002) that scikit-image's
//                    unwrap_phase implements.  Processing the grid edges in
//                    ascending reliability order, joining groups and
//                    shifting the joined group by whole turns, is Kruskal's
//                    algorithm: the edges that join groups form the minimum
//                    spanning tree of the edge weights, and every pixel's
//                    unwrapped value is its wrapped value plus the turns
//                    accumulated along the tree path from the pixel that
//                    heads the final group.  The GPU builds the same tree
//                    with Boruvka rounds (each component hooks onto its
//                    lightest outgoing edge; ties broken by the edge index,
//                    a strict total order, so no cycles) and carries the
//                    turn offsets through weighted pointer jumping:
//                      k_uw_init     pixel reliabilities (FP64), identity
//                      k_uw_minw     lightest outgoing edge weight per root
//                      k_uw_mine     its lowest edge index
//                      k_uw_hook     root -> neighbouring root, turn offset
//                      k_uw_jump     pointer jumping among this round's roots
//                      k_uw_flatten  every pixel -> its new root
//                    (at most ceil(log2(pixels)) + 2 rounds; a round with no
//                    hook ends the work of the following ones), with
//                      k_uw_anchor   first edge of each frame (after round 0's
//                                    k_uw_mine), then
//                      k_uw_finish   phi + 2 pi k, k relative to pixel 1 of
//                                    the frame's first edge
//   align            k_phase_min (global minimum), k_align (one CTA: the
//                    five border samples unwrapped along the angle axis,
//                    per-angle majority step, whole turns of the minimum)
//   k_compose        phi - remove[a]; rytov output u0 * (1j * phi + lna)
//                    with NumPy's complex arithmetic, radon output phi
// ODT_SINO_UNWRAP takes a real wrapped phase and skips k_phase;
// ODT_SINO_ALIGN takes an unwrapped real phase and runs the last three steps.
//
// Every wait is bounded: k_uw_jump's loop stops after a fixed number of
// steps and records ODT_ERR_DEVICE_CHECK in the status word.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>

#include "../../include/odtbrain_gb300.h"
#include "odt_internal.cuh"

namespace odt {
namespace {

constexpr double PI_D = 3.14159265358979323846;
constexpr double TWOPI_D = 2.0 * 3.14159265358979323846;
constexpr double BORDER_BASE = 9999999.0;
constexpr unsigned long long NONE64 = ~0ull;
constexpr uint32_t NONE32 = ~0u;
constexpr int JUMP_LIMIT = 1 << 22;
constexpr int STATUS_JUMP = 1, STATUS_SPLIT = 2;

template <class T>
struct C2 {
    T x, y;
};

// ---- exact (non-contracted) arithmetic in T -------------------------------
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }

// a / b for complex numbers, Smith's algorithm (R. L. Smith, "Algorithm
// 116: Complex division", CACM 5(8), 1962), the form NumPy uses.
template <class T>
__device__ __forceinline__ C2<T> cdiv_smith(C2<T> a, C2<T> b)
{
    const T br = fabs(b.x), bi = fabs(b.y);
    C2<T> r;
    if (br >= bi) {
        if (br == T(0) && bi == T(0)) {
            r.x = div_rn(a.x, br);
            r.y = div_rn(a.y, br);
        } else {
            const T rat = div_rn(b.y, b.x);
            const T scl = div_rn(T(1), add_rn(b.x, mul_rn(b.y, rat)));
            r.x = mul_rn(add_rn(a.x, mul_rn(a.y, rat)), scl);
            r.y = mul_rn(sub_rn(a.y, mul_rn(a.x, rat)), scl);
        }
    } else {
        const T rat = div_rn(b.x, b.y);
        const T scl = div_rn(T(1), add_rn(b.y, mul_rn(b.x, rat)));
        r.x = mul_rn(add_rn(mul_rn(a.x, rat), a.y), scl);
        r.y = mul_rn(sub_rn(mul_rn(a.y, rat), a.x), scl);
    }
    return r;
}

// a * b, NumPy's complex product (re = ar*br - ai*bi, im = ar*bi + ai*br).
template <class T>
__device__ __forceinline__ C2<T> cmul_np(C2<T> a, C2<T> b)
{
    C2<T> r;
    r.x = sub_rn(mul_rn(a.x, b.x), mul_rn(a.y, b.y));
    r.y = add_rn(mul_rn(a.x, b.y), mul_rn(a.y, b.x));
    return r;
}

// NumPy's floating-point remainder with the sign of the divisor (b > 0).
template <class T>
__device__ __forceinline__ T np_mod_pos(T a, T b)
{
    T m = fmod(a, b);
    if (m != T(0)) {
        if (m < T(0))
            m = add_rn(m, b);
    } else {
        m = T(0);
    }
    return m;
}

// NumPy's floor quotient of divmod(a, b) (b > 0).
template <class T>
__device__ __forceinline__ T np_floordiv(T a, T b)
{
    T m = fmod(a, b);
    T div = div_rn(sub_rn(a, m), b);
    if (m != T(0)) {
        if ((b < T(0)) != (m < T(0)))
            div = sub_rn(div, T(1));
    }
    T fl;
    if (div != T(0)) {
        fl = floor(div);
        if (sub_rn(div, fl) > T(0.5))
            fl = add_rn(fl, T(1));
    } else {
        fl = copysign(T(0), div_rn(a, b));
    }
    return fl;
}

// ---- packed (parent, turn offset) words -----------------------------------
__device__ __forceinline__ unsigned long long pack(uint32_t par, int32_t off)
{
    return ((unsigned long long)par << 32) | (uint32_t)off;
}
__device__ __forceinline__ uint32_t par_of(unsigned long long w) { return (uint32_t)(w >> 32); }
__device__ __forceinline__ int32_t off_of(unsigned long long w) { return (int32_t)(uint32_t)(w & 0xffffffffull); }

__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// Pseudo-random border value in [0, 2^31): splitmix64 finaliser of
// seed * 0x9E3779B97F4A7C15 + (n + 1) * 0xBF58476D1CE4E5B9.
__device__ __forceinline__ double border_noise(uint32_t seed, unsigned long long n)
{
    unsigned long long x = (unsigned long long)seed * 0x9E3779B97F4A7C15ull + (n + 1ull) * 0xBF58476D1CE4E5B9ull;
    x ^= x >> 30;
    x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27;
    x *= 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (double)(long long)(x >> 33);
}

__device__ __forceinline__ double wrapd(double d)
{
    if (d > PI_D)
        return __dsub_rn(d, TWOPI_D);
    if (d < -PI_D)
        return __dadd_rn(d, TWOPI_D);
    return d;
}

// Frame geometry for the unwrap kernels: frame a, row i, column j of global
// pixel p; local edge index: horizontal (i, j)-(i, j+1) at i*(W-1)+j, then
// vertical (i, j)-(i+1, j) at H*(W-1) + i*W + j.
struct Frames {
    int H, W;
    long long P;  // H * W
    long long N;  // A * P
};

// The per-pixel kernels run on blocks of 32 x 8 pixels over a grid
// (ceil(W/32), ceil(H/8), frames): frame, row and column come from the
// block and thread indices (no divisions); p = (a*H + i)*W + j < 2^31.
struct Px {
    int a, i, j;
    uint32_t p;
    bool ok;
};
__device__ __forceinline__ Px pixel(const Frames &F)
{
    Px x;
    x.j = (int)(blockIdx.x * 32 + threadIdx.x);
    x.i = (int)(blockIdx.y * 8 + threadIdx.y);
    x.a = (int)blockIdx.z;
    x.ok = x.i < F.H && x.j < F.W;
    x.p = ((uint32_t)x.a * (uint32_t)F.H + (uint32_t)x.i) * (uint32_t)F.W + (uint32_t)x.j;
    return x;
}

__device__ __forceinline__ void edge_ends(const Frames &F, uint32_t base, uint32_t le, uint32_t &u, uint32_t &v)
{
    const uint32_t nh = (uint32_t)F.H * (uint32_t)(F.W - 1);
    if (le < nh) {
        const uint32_t i = le / (uint32_t)(F.W - 1), j = le - i * (uint32_t)(F.W - 1);
        u = base + i * (uint32_t)F.W + j;
        v = u + 1;
    } else {
        const uint32_t l2 = le - nh;
        u = base + l2;
        v = u + (uint32_t)F.W;
    }
}

// ---------------------------------------------------------------------------
template <class T>
__global__ void k_phase(const C2<T> *sino, const C2<T> *u0arr, C2<T> u0s, long long n, int rytov, T *phi,
                        C2<T> *out)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        C2<T> q = sino[i];
        if (rytov) {
            q = cdiv_smith<T>(q, u0arr ? u0arr[i] : u0s);
            out[i].x = log(hypot(q.x, q.y));
        }
        phi[i] = atan2(q.y, q.x);
    }
}

// numpy.unwrap along each line of `len` values (period 2 pi, discont pi), in
// T arithmetic and NumPy's order: dd = p[i] - p[i-1];
// ddmod = mod(dd + pi, 2 pi) - pi, set to +pi where ddmod == -pi and dd > 0;
// correction ddmod - dd (0 where |dd| < pi), accumulated sequentially.
template <class T>
__device__ __forceinline__ void unwrap_line(T *p, long long len, long long stride, double *steps_out)
{
    const T pi = (T)PI_D, twopi = (T)TWOPI_D;
    T prev = p[0];
    T cum = T(0);
    if (steps_out)
        steps_out[0] = (double)sub_rn(prev, prev);
    for (long long i = 1; i < len; ++i) {
        const T cur = p[i * stride];
        const T dd = sub_rn(cur, prev);
        T ddmod = add_rn(np_mod_pos<T>(add_rn(dd, pi), twopi), -pi);
        if (ddmod == -pi && dd > T(0))
            ddmod = pi;
        T pc = sub_rn(ddmod, dd);
        if (fabs(dd) < pi)
            pc = T(0);
        cum = add_rn(cum, pc);
        const T up = add_rn(cur, cum);
        if (steps_out)
            steps_out[i] = (double)sub_rn(cur, up);  // sample - unwrapped
        else
            p[i * stride] = up;
        prev = cur;
    }
}

template <class T>
__global__ void k_unwrap_rows(T *phi, long long rows, int len)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows)
        unwrap_line<T>(phi + r * len, len, 1, nullptr);
}

// ---- 3D frames: reliability-sorted unwrapping as a Boruvka MST ------------
// Warp-aggregated append to a list: every lane of the warp must call it (with
// want = false where it has nothing to add); returns the slot of a wanting
// lane.
__device__ __forceinline__ uint32_t append_slot(uint32_t *cnt, bool want)
{
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (mask) {
        const int leader = __ffs(mask) - 1;
        if (lane == leader)
            base = atomicAdd(cnt, (uint32_t)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

// Root of pixel p and p's turns relative to it: follow the (parent, offset)
// words until a root (a word pointing to itself); then store the result in
// p's word (path compression; the words of pixels only ever move to a root
// of the same component).  Bounded: gives up with STATUS_JUMP.
__device__ __forceinline__ uint32_t resolve(unsigned long long *word, uint32_t p, int32_t &off, uint32_t *status)
{
    const unsigned long long w = __ldcg(word + p);
    uint32_t x = par_of(w);
    int32_t acc = off_of(w);
    int hops = 0;
    for (;;) {
        const unsigned long long wx = __ldcg(word + x);
        if (par_of(wx) == x)
            break;
        acc += off_of(wx);
        x = par_of(wx);
        if (++hops > JUMP_LIMIT) {
            atomicOr(status, STATUS_JUMP);
            break;
        }
    }
    if (hops > 0)
        __stcg(word + p, pack(x, acc));
    off = acc;
    return x;
}

// Pixel reliabilities.  A 32 x 8 block stages its tile of phases (plus a
// one-pixel halo) as doubles in shared memory and forms each wrapped first
// difference once -- right, down, down-right and down-left of every tile
// position -- so an interior pixel's second differences
//   H = wrap(l - c) - wrap(c - r), V (up/down), D1 (up-left/down-right),
//   D2 (up-right/down-left)
// are differences of those (the same FP64 operands and operations as the
// direct formula, so the values are identical).  Border pixels get
// 9999999 + border_noise.
constexpr int UI_TW = 34, UI_TH = 10;  // tile with halo

template <class T>
__global__ void __launch_bounds__(256) k_uw_init(const T *phi, Frames F, uint32_t seed, double *rel,
                                                 unsigned long long *word, unsigned long long *bw, uint32_t *be)
{
    __shared__ double ph[UI_TH][UI_TW];
    __shared__ double dR[UI_TH][UI_TW], dD[UI_TH][UI_TW], dDR[UI_TH][UI_TW], dDL[UI_TH][UI_TW];
    const Px x = pixel(F);
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int i0 = (int)blockIdx.y * 8 - 1, j0 = (int)blockIdx.x * 32 - 1;
    const T *frame = phi + (size_t)x.a * (size_t)F.P;
    for (int t = tid; t < UI_TH * UI_TW; t += 256) {
        const int ti = t / UI_TW, tj = t - ti * UI_TW;
        const int gi = i0 + ti, gj = j0 + tj;
        ph[ti][tj] = (gi >= 0 && gi < F.H && gj >= 0 && gj < F.W) ? (double)frame[(size_t)gi * F.W + gj] : 0.0;
    }
    __syncthreads();
    for (int t = tid; t < UI_TH * UI_TW; t += 256) {
        const int ti = t / UI_TW, tj = t - ti * UI_TW;
        const double c = ph[ti][tj];
        if (tj + 1 < UI_TW)
            dR[ti][tj] = wrapd(__dsub_rn(c, ph[ti][tj + 1]));
        if (ti + 1 < UI_TH) {
            dD[ti][tj] = wrapd(__dsub_rn(c, ph[ti + 1][tj]));
            if (tj + 1 < UI_TW)
                dDR[ti][tj] = wrapd(__dsub_rn(c, ph[ti + 1][tj + 1]));
            if (tj >= 1)
                dDL[ti][tj] = wrapd(__dsub_rn(c, ph[ti + 1][tj - 1]));
        }
    }
    __syncthreads();
    if (!x.ok)
        return;
    const uint32_t p = x.p;
    const int i = x.i, j = x.j;
    double r;
    if (i >= 1 && i <= F.H - 2 && j >= 1 && j <= F.W - 2) {
        const int ti = threadIdx.y + 1, tj = threadIdx.x + 1;
        const double h = __dsub_rn(dR[ti][tj - 1], dR[ti][tj]);         // wrap(l - c) - wrap(c - r)
        const double v = __dsub_rn(dD[ti - 1][tj], dD[ti][tj]);         // wrap(u - c) - wrap(c - d)
        const double d1 = __dsub_rn(dDR[ti - 1][tj - 1], dDR[ti][tj]);  // wrap(ul - c) - wrap(c - dr)
        const double d2 = __dsub_rn(dDL[ti - 1][tj + 1], dDL[ti][tj]);  // wrap(ur - c) - wrap(c - dl)
        r = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(h, h), __dmul_rn(v, v)), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
    } else {
        r = __dadd_rn(BORDER_BASE, border_noise(seed, (unsigned long long)((uint32_t)i * (uint32_t)F.W + j)));
    }
    rel[p] = r;
    word[p] = pack(p, 0);
    bw[p] = NONE64;
    be[p] = NONE32;
}

// Lightest outgoing edge weight of every component root (edges handled by
// their pixel 1: right and down neighbours).
// Lightest outgoing edge weight of every component root (edges handled by
// their pixel 1: right and down neighbours).  With `elist`, the crossing
// edges are also appended to it as (pixel 1, frame-local edge index).
__global__ void k_uw_minw(Frames F, const double *rel, const unsigned long long *word, unsigned long long *bw,
                          const uint32_t *flags, int round, uint2 *elist, uint32_t *ecnt)
{
    if (round > 0 && flags[round - 1] == 0)
        return;
    const Px x = pixel(F);
    const uint32_t p = x.p;
    const int i = x.i, j = x.j;
    const uint32_t rp = x.ok ? par_of(word[p]) : 0u;
    const double relp = x.ok ? rel[p] : 0.0;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        bool cross = false;
        uint32_t le = 0;
        if (x.ok && (d == 0 ? (j + 1 < F.W) : (i + 1 < F.H))) {
            const uint32_t q = p + (d == 0 ? 1u : (uint32_t)F.W);
            const uint32_t rq = par_of(word[q]);
            if (rp != rq) {
                cross = true;
                le = d == 0 ? (uint32_t)(i * (F.W - 1) + j)
                            : (uint32_t)(F.H * (F.W - 1)) + (uint32_t)i * (uint32_t)F.W + (uint32_t)j;
                const unsigned long long wb = dbits(__dadd_rn(relp, rel[q]));
                if (wb < bw[rp])
                    atomicMin(bw + rp, wb);
                if (wb < bw[rq])
                    atomicMin(bw + rq, wb);
            }
        }
        if (elist) {
            // list entry: (pixel 1, local edge index | vertical flag)
            const uint32_t slot = append_slot(ecnt, cross);
            if (cross)
                elist[slot] = make_uint2(p, d == 0 ? le : (le | 0x80000000u));
        }
    }
}

// Lowest edge index among each root's lightest outgoing edges.
__global__ void k_uw_mine(Frames F, const double *rel, const unsigned long long *word, const unsigned long long *bw,
                          uint32_t *be, const uint32_t *flags, int round)
{
    if (round > 0 && flags[round - 1] == 0)
        return;
    const Px x = pixel(F);
    if (!x.ok)
        return;
    const uint32_t p = x.p;
    const int i = x.i, j = x.j;
    const uint32_t lp = (uint32_t)i * (uint32_t)F.W + (uint32_t)j;
    const uint32_t rp = par_of(word[p]);
    const double relp = rel[p];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        if (d == 0 ? (j + 1 >= F.W) : (i + 1 >= F.H))
            continue;
        const uint32_t q = p + (d == 0 ? 1u : (uint32_t)F.W);
        const uint32_t rq = par_of(word[q]);
        if (rp == rq)
            continue;
        const unsigned long long wb = dbits(__dadd_rn(relp, rel[q]));
        const uint32_t le = d == 0 ? (uint32_t)(i * (F.W - 1) + j) : (uint32_t)(F.H * (F.W - 1)) + lp;
        if (wb == bw[rp])
            atomicMin(be + rp, le);
        if (wb == bw[rq])
            atomicMin(be + rq, le);
    }
}

// Every root hooks onto the root across its chosen edge, except the lower
// root of a pair that chose the same edge.  rw[r] = (new parent, turns of r
// relative to it); written for every root.
template <class T>
__global__ void k_uw_hook(Frames F, const T *phi, const unsigned long long *word, const uint32_t *be,
                          unsigned long long *rw, uint32_t *flags, int round, uint32_t *rlist, uint32_t *rcnt)
{
    if (round > 0 && flags[round - 1] == 0)
        return;
    const Px x = pixel(F);
    const uint32_t r = x.p;
    bool keep = false;  // a root after this round with an outgoing edge left
    if (x.ok && par_of(word[r]) == r) {
        const uint32_t le = be[r];
        if (le == NONE32) {
            rw[r] = pack(r, 0);
        } else {
            const uint32_t base = (uint32_t)x.a * (uint32_t)F.P;
            uint32_t u, v;
            edge_ends(F, base, le, u, v);
            const unsigned long long wu = word[u], wv = word[v];
            const bool u_in_r = par_of(wu) == r;
            const uint32_t s = u_in_r ? par_of(wv) : par_of(wu);
            if (be[s] == le && r < s) {
                rw[r] = pack(r, 0);
                keep = true;
            } else {
                // turns: k(v) - k(u) = -e with e = +1 / -1 / 0 as
                // phi[u] - phi[v] is below -pi / above pi / neither (the
                // reference's find_wrap)
                const double d = (double)phi[u] - (double)phi[v];
                const int e = d > PI_D ? -1 : (d < -PI_D ? 1 : 0);
                const int32_t ou = off_of(wu), ov = off_of(wv);
                rw[r] = pack(s, u_in_r ? (e + ov - ou) : (-e + ou - ov));
                flags[round] = 1;
            }
        }
    }
    if (rlist) {
        const uint32_t slot = append_slot(rcnt, keep);
        if (keep)
            rlist[slot] = r;
    }
}

__global__ void k_uw_jump(Frames F, const unsigned long long *word, unsigned long long *rw, uint32_t *flags,
                          int round, uint32_t *status)
{
    if (flags[round] == 0)
        return;
    const Px x = pixel(F);
    if (!x.ok)
        return;
    const uint32_t r = x.p;
    if (par_of(word[r]) != r)
        return;
    unsigned long long w = __ldcg(rw + r);
    for (int it = 0;; ++it) {
        const uint32_t pp = par_of(w);
        if (pp == r)
            break;
        const unsigned long long wp = __ldcg(rw + pp);
        if (par_of(wp) == pp)
            break;
        w = pack(par_of(wp), off_of(w) + off_of(wp));
        __stcg(rw + r, w);
        if (it >= JUMP_LIMIT) {
            atomicOr(status, STATUS_JUMP);
            break;
        }
    }
}

__global__ void k_uw_flatten(Frames F, unsigned long long *word, const unsigned long long *rw,
                             unsigned long long *bw, uint32_t *be, const uint32_t *flags, int round)
{
    if (flags[round] == 0)
        return;
    const Px x = pixel(F);
    if (!x.ok)
        return;
    const uint32_t p = x.p;
    const unsigned long long w = word[p];
    const unsigned long long wr = rw[par_of(w)];
    word[p] = pack(par_of(wr), off_of(w) + off_of(wr));
    bw[p] = NONE64;
    be[p] = NONE32;
}

// ---- rounds >= 2 on lists ---------------------------------------------------
// From round 2 on, only the edges that crossed components in the previous
// round and the roots that are left are visited (lists compacted every
// round); pixel roots are found by following the (parent, offset) words,
// which only the roots update (k_ul_update), with path compression.  Grids
// are fixed; the kernels stride over the device-side counts.
constexpr int UL_GRID = 152 * 8, UL_BLOCK = 256;

__global__ void __launch_bounds__(UL_BLOCK) k_ul_edges_w(const double *rel, unsigned long long *word,
                                                         unsigned long long *bw, const uint2 *ein,
                                                         const uint32_t *ecnt_in, uint2 *eout, uint32_t *ecnt_out,
                                                         int W, const uint32_t *flags, int round, uint32_t *status)
{
    if (flags[round - 1] == 0)
        return;
    const uint32_t n = *ecnt_in;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const uint32_t k = b + threadIdx.x;
        bool cross = false;
        uint2 e = make_uint2(0, 0);
        if (k < n) {
            e = ein[k];
            const uint32_t u = e.x;
            const uint32_t v = u + ((e.y & 0x80000000u) ? (uint32_t)W : 1u);
            int32_t ou, ov;
            const uint32_t ru = resolve(word, u, ou, status), rv = resolve(word, v, ov, status);
            if (ru != rv) {
                cross = true;
                const unsigned long long wb = dbits(__dadd_rn(rel[u], rel[v]));
                if (wb < bw[ru])
                    atomicMin(bw + ru, wb);
                if (wb < bw[rv])
                    atomicMin(bw + rv, wb);
            }
        }
        const uint32_t slot = append_slot(ecnt_out, cross);
        if (cross)
            eout[slot] = e;
    }
}

__global__ void __launch_bounds__(UL_BLOCK) k_ul_edges_e(const double *rel, unsigned long long *word,
                                                         const unsigned long long *bw, uint32_t *be, const uint2 *el,
                                                         const uint32_t *ecnt, int W, const uint32_t *flags,
                                                         int round, uint32_t *status)
{
    if (flags[round - 1] == 0)
        return;
    const uint32_t n = *ecnt;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint2 e = el[k];
        const uint32_t u = e.x;
        const uint32_t v = u + ((e.y & 0x80000000u) ? (uint32_t)W : 1u);
        const uint32_t le = e.y & 0x7fffffffu;
        int32_t ou, ov;
        const uint32_t ru = resolve(word, u, ou, status), rv = resolve(word, v, ov, status);
        if (ru == rv)
            continue;
        const unsigned long long wb = dbits(__dadd_rn(rel[u], rel[v]));
        if (wb == bw[ru])
            atomicMin(be + ru, le);
        if (wb == bw[rv])
            atomicMin(be + rv, le);
    }
}

template <class T>
__global__ void __launch_bounds__(UL_BLOCK) k_ul_hook(Frames F, const T *phi, unsigned long long *word,
                                                      const uint32_t *be, unsigned long long *rw, const uint32_t *rin,
                                                      const uint32_t *rcnt_in, uint32_t *rout, uint32_t *rcnt_out,
                                                      uint32_t *flags, int round, uint32_t *status)
{
    if (flags[round - 1] == 0)
        return;
    const uint32_t n = *rcnt_in;
    for (uint32_t b = blockIdx.x * blockDim.x; b < n; b += gridDim.x * blockDim.x) {
        const uint32_t k = b + threadIdx.x;
        bool keep = false;
        uint32_t r = 0;
        if (k < n) {
            r = rin[k];
            const uint32_t le = be[r];
            if (le == NONE32) {
                rw[r] = pack(r, 0);
            } else {
                const uint32_t base = r / (uint32_t)F.P * (uint32_t)F.P;
                uint32_t u, v;
                edge_ends(F, base, le, u, v);
                int32_t ou, ov;
                const uint32_t ru = resolve(word, u, ou, status), rv = resolve(word, v, ov, status);
                const bool u_in_r = ru == r;
                const uint32_t s = u_in_r ? rv : ru;
                if (be[s] == le && r < s) {
                    rw[r] = pack(r, 0);
                    keep = true;
                } else {
                    const double d = (double)phi[u] - (double)phi[v];
                    const int e = d > PI_D ? -1 : (d < -PI_D ? 1 : 0);
                    rw[r] = pack(s, u_in_r ? (e + ov - ou) : (-e + ou - ov));
                    flags[round] = 1;
                }
            }
        }
        const uint32_t slot = append_slot(rcnt_out, keep);
        if (keep)
            rout[slot] = r;
    }
}

__global__ void __launch_bounds__(UL_BLOCK) k_ul_jump(unsigned long long *rw, const uint32_t *rl, const uint32_t *rcnt,
                                                      const uint32_t *flags, int round, uint32_t *status)
{
    if (flags[round] == 0)
        return;
    const uint32_t n = *rcnt;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t r = rl[k];
        unsigned long long w = __ldcg(rw + r);
        for (int it = 0;; ++it) {
            const uint32_t pp = par_of(w);
            if (pp == r)
                break;
            const unsigned long long wp = __ldcg(rw + pp);
            if (par_of(wp) == pp)
                break;
            w = pack(par_of(wp), off_of(w) + off_of(wp));
            __stcg(rw + r, w);
            if (it >= JUMP_LIMIT) {
                atomicOr(status, STATUS_JUMP);
                break;
            }
        }
    }
}

// the roots of this round take their new parent word; per-root minima reset
__global__ void __launch_bounds__(UL_BLOCK) k_ul_update(unsigned long long *word, const unsigned long long *rw,
                                                        unsigned long long *bw, uint32_t *be, const uint32_t *rl,
                                                        const uint32_t *rcnt, const uint32_t *flags, int round)
{
    if (flags[round] == 0)
        return;
    const uint32_t n = *rcnt;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t r = rl[k];
        word[r] = rw[r];
        bw[r] = NONE64;
        be[r] = NONE32;
    }
}

// First edge of each frame in (weight, index) order, whose pixel 1 starts
// the first group: after round 0's k_uw_mine every pixel holds its lightest
// incident edge (bw, be), so the frame's first edge is the lexicographic
// minimum of those pairs.  One CTA per frame, no atomics.
__global__ void __launch_bounds__(1024) k_uw_anchor(Frames F, const unsigned long long *bw, const uint32_t *be,
                                                    uint32_t *fe)
{
    __shared__ unsigned long long sw[32];
    __shared__ uint32_t se[32];
    const long long a = blockIdx.x;
    const long long base = a * F.P;
    unsigned long long mw = NONE64;
    uint32_t me = NONE32;
    for (long long lp = threadIdx.x; lp < F.P; lp += blockDim.x) {
        const unsigned long long w = bw[base + lp];
        const uint32_t e = be[base + lp];
        if (w < mw || (w == mw && e < me)) {
            mw = w;
            me = e;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, mw, o);
        const uint32_t e = __shfl_xor_sync(0xffffffffu, me, o);
        if (w < mw || (w == mw && e < me)) {
            mw = w;
            me = e;
        }
    }
    const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        sw[wid] = mw;
        se[wid] = me;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < nw; ++i)
            if (sw[i] < mw || (sw[i] == mw && se[i] < me)) {
                mw = sw[i];
                me = se[i];
            }
        fe[a] = me;
    }
}

template <class T>
__global__ void k_uw_finish(Frames F, T *phi, unsigned long long *word, const uint32_t *fe, uint32_t *status)
{
    const Px x = pixel(F);
    if (!x.ok)
        return;
    const uint32_t p = x.p;
    const int a = x.a;
    int32_t op;
    const uint32_t rp = resolve(word, p, op, status);
    int32_t ka = 0;
    if (fe[a] != NONE32) {
        uint32_t u, v;
        edge_ends(F, (uint32_t)a * (uint32_t)F.P, fe[a], u, v);
        const uint32_t ra = resolve(word, u, ka, status);
        if (ra != rp) {
            atomicOr(status, STATUS_SPLIT);
            return;
        }
    }
    const int32_t k = op - ka;
    if (k != 0)
        phi[p] = (T)__dadd_rn((double)phi[p], __dmul_rn(TWOPI_D, (double)k));
}

// ---- align_unwrapped -------------------------------------------------------
// Order-preserving unsigned keys of T (NaN handled separately).
__device__ __forceinline__ unsigned long long okey(double v)
{
    const unsigned long long b = dbits(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double okey_val(unsigned long long k)
{
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

template <class T>
__global__ void k_phase_min(const T *phi, long long n, unsigned long long *minkey, uint32_t *nan_seen)
{
    unsigned long long m = NONE64;
    bool nan = false;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = (double)phi[i];
        if (v != v)
            nan = true;
        else
            m = min(m, okey(v));
    }
    for (int o = 16; o > 0; o >>= 1)
        m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m != NONE64)
        atomicMin(minkey, m);
    if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0)
        atomicOr(nan_seen, 1u);
}

// One CTA.  steps[i][a] = sample_i[a] - unwrap(sample_i)[a] for the five
// border samples; remove[a] = mode_i(steps[i][a]) (most frequent value, the
// smallest among equally frequent ones) + whole turns of the global minimum
// (divmod with the remainder closest to zero).
template <class T>
__global__ void k_align(const T *phi, long long A, int ny, int nx, int three_d, const unsigned long long *minkey,
                        const uint32_t *nan_seen, double *steps, double *remove)
{
    const long long fr = three_d ? (long long)ny * nx : nx;
    if (threadIdx.x < 5) {
        long long off;
        const int s = threadIdx.x;
        if (three_d) {
            const long long last = (long long)(ny - 1) * nx;
            const long long offs[5] = {0, nx - 1, last, last + nx - 1, 1};
            off = offs[s];
        } else {
            const long long offs[5] = {0, 1, 2, nx - 1, nx - 2};
            off = offs[s];
        }
        unwrap_line<T>(const_cast<T *>(phi) + off, A, fr, steps + s * A);
    }
    __syncthreads();
    // whole turns of the minimum, in T like the reference's scalar divmod
    double shift;
    if (*nan_seen) {
        shift = __longlong_as_double(0x7ff8000000000000ll);
    } else {
        const T mn = (T)okey_val(*minkey);
        const T twopi = (T)TWOPI_D;
        T q = np_floordiv<T>(mn, twopi);
        const T rm = np_mod_pos<T>(mn, twopi);
        const T sr = rm > T(0) ? T(1) : (rm < T(0) ? T(-1) : T(0));
        if (fabs(rm) > (T)PI_D)
            q = add_rn(q, sr);
        shift = (double)mul_rn(q, twopi);
    }
    for (long long a = threadIdx.x; a < A; a += blockDim.x) {
        double v[5];
#pragma unroll
        for (int i = 0; i < 5; ++i)
            v[i] = steps[i * A + a];
        double best = 0.0;
        int bestc = 0;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            int c = 0;
#pragma unroll
            for (int k = 0; k < 5; ++k)
                c += v[k] == v[i];
            if (c > bestc || (c == bestc && v[i] < best)) {
                bestc = c;
                best = v[i];
            }
        }
        remove[a] = __dadd_rn(best, shift);
    }
}

// grid (x, angle): the angle is blockIdx.y, no division per sample
template <class T>
__global__ void k_compose(const T *phi, const double *remove, long long per_angle, long long n, int rytov,
                          const C2<T> *u0arr, C2<T> u0s, C2<T> *outc, T *outr)
{
    const long long a = blockIdx.y;
    const double rm = remove ? remove[a] : 0.0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < per_angle;
         k += (long long)gridDim.x * blockDim.x) {
        const long long i = a * per_angle + k;
        T ph = phi[i];
        if (remove)
            ph = (T)__dsub_rn((double)ph, rm);
        if (!rytov) {
            outr[i] = ph;
            continue;
        }
        // 1j * phi + lna, then u0 * (...), NumPy's complex arithmetic
        const T lna = outc[i].x;
        C2<T> z;
        z.x = add_rn(sub_rn(mul_rn(T(0), ph), mul_rn(T(1), T(0))), lna);
        z.y = add_rn(add_rn(mul_rn(T(0), T(0)), mul_rn(T(1), ph)), T(0));
        outc[i] = cmul_np<T>(u0arr ? u0arr[i] : u0s, z);
    }
}

// ---------------------------------------------------------------------------
struct Layout {
    size_t phi, rel, word, rw, bw, be, fe, flags, status, minkey, nan, steps, remove, elist[2], rlist[2], cnt, total;
};

int num_rounds(long long P)
{
    int r = 1;
    while ((1ll << (r - 1)) < P)
        ++r;
    return r + 1;
}

Layout layout_of(const odt_sino_desc &d)
{
    const bool c128 = d.dtype == ODT_DATA_C128 || d.dtype == ODT_DATA_F64;
    const long long A = d.num_angles;
    const long long P = d.ny > 0 ? (long long)d.ny * d.nx : (long long)d.nx;
    const long long N = A * P;
    const bool three_d = d.ny > 0 && d.kind != ODT_SINO_ALIGN;  // unwrap buffers
    Layout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += (bytes + 255) / 256 * 256;
        return at;
    };
    L.status = take(4);
    L.minkey = take(8);
    L.nan = take(4);
    L.phi = take((size_t)N * (c128 ? 8 : 4));
    L.steps = take((size_t)5 * A * 8);
    L.remove = take((size_t)A * 8);
    if (three_d) {
        L.flags = take((size_t)(num_rounds(P) + 1) * 4);
        L.rel = take((size_t)N * 8);
        L.word = take((size_t)N * 8);
        L.rw = take((size_t)N * 8);
        L.bw = take((size_t)N * 8);
        L.be = take((size_t)N * 4);
        L.fe = take((size_t)A * 4);
        for (int k = 0; k < 2; ++k) {
            L.elist[k] = take((size_t)N * 2 * 8);
            L.rlist[k] = take((size_t)N * 4);
        }
        L.cnt = take(4 * 4);
    }
    L.total = o;
    return L;
}

odt_status check_desc(const odt_sino_desc *d)
{
    if (!d)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL descriptor");
    if (d->num_angles < 1 || d->nx < 1 || d->ny < 0)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "sinogram sizes must be positive");
    if (d->kind < ODT_SINO_RYTOV || d->kind > ODT_SINO_UNWRAP)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "unknown sinogram conversion");
    const bool real_in = d->kind == ODT_SINO_ALIGN || d->kind == ODT_SINO_UNWRAP;
    if (real_in ? (d->dtype != ODT_DATA_F32 && d->dtype != ODT_DATA_F64)
                : (d->dtype != ODT_DATA_C64 && d->dtype != ODT_DATA_C128))
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, real_in
                                                                   ? "phase dtype must be float32 or float64"
                                                                   : "sinogram dtype must be complex64 or complex128");
    if (d->kind == ODT_SINO_ALIGN && !d->align)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "alignment-only call without align");
    const long long P = d->ny > 0 ? (long long)d->ny * d->nx : (long long)d->nx;
    if (d->num_angles > (1ll << 31) / P)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "sinogram too large (more than 2^31 samples)");
    if (d->num_angles > 65535)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "more than 65535 angles");
    if (d->align && d->ny == 0 && d->nx < 3)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "alignment needs at least 3 detector columns");
    if (d->align && d->ny > 0 && d->nx < 2)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "alignment needs at least 2 detector columns");
    return ODT_OK;
}

odt_status launched(const char *what)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return (odt_status)set_error(ODT_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
    return ODT_OK;
}

template <class T>
odt_status run(const odt_sino_desc &d, const void *sino, void *out, char *ws, cudaStream_t s)
{
    const Layout L = layout_of(d);
    const bool three_d = d.ny > 0;
    const bool real_in = d.kind == ODT_SINO_ALIGN || d.kind == ODT_SINO_UNWRAP;
    const bool unwrap = d.kind != ODT_SINO_ALIGN;
    const long long A = d.num_angles;
    const long long P = three_d ? (long long)d.ny * d.nx : (long long)d.nx;
    const long long N = A * P;
    const bool rytov = d.kind == ODT_SINO_RYTOV;
    T *phi = (T *)(ws + L.phi);
    uint32_t *status = (uint32_t *)(ws + L.status);
    C2<T> u0s;
    u0s.x = (T)d.u0_re;
    u0s.y = (T)d.u0_im;
    const C2<T> *u0arr = (const C2<T> *)d.u0;
    C2<T> *outc = rytov ? (C2<T> *)out : nullptr;
    T *outr = rytov ? nullptr : (T *)out;
    if (cudaMemsetAsync(ws, 0, L.phi, s) != cudaSuccess)
        return launched("sinogram workspace reset");
    const unsigned eg = (unsigned)std::min<long long>((N + 255) / 256, 152ll * 16);
    if (real_in) {
        if (cudaMemcpyAsync(phi, sino, (size_t)N * sizeof(T), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return launched("phase copy");
    } else {
        k_phase<T><<<eg, 256, 0, s>>>((const C2<T> *)sino, u0arr, u0s, N, rytov ? 1 : 0, phi, outc);
    }
    if (!unwrap) {
    } else if (!three_d) {
        k_unwrap_rows<T><<<(unsigned)((A + 127) / 128), 128, 0, s>>>(phi, A, d.nx);
    } else {
        Frames F{d.ny, d.nx, P, N};
        double *rel = (double *)(ws + L.rel);
        unsigned long long *word = (unsigned long long *)(ws + L.word);
        unsigned long long *rw = (unsigned long long *)(ws + L.rw);
        unsigned long long *bw = (unsigned long long *)(ws + L.bw);
        uint32_t *be = (uint32_t *)(ws + L.be);
        uint32_t *fe = (uint32_t *)(ws + L.fe);
        uint32_t *flags = (uint32_t *)(ws + L.flags);
        const int rounds = num_rounds(P);
        if (cudaMemsetAsync(flags, 0, (size_t)(rounds + 1) * 4, s) != cudaSuccess)
            return launched("unwrap workspace reset");
        const dim3 pg((unsigned)((d.nx + 31) / 32), (unsigned)((d.ny + 7) / 8), (unsigned)A), pb(32, 8);
        uint2 *el[2] = {(uint2 *)(ws + L.elist[0]), (uint2 *)(ws + L.elist[1])};
        uint32_t *rl[2] = {(uint32_t *)(ws + L.rlist[0]), (uint32_t *)(ws + L.rlist[1])};
        uint32_t *ecnt = (uint32_t *)(ws + L.cnt), *rcnt = ecnt + 2;
        if (cudaMemsetAsync(ecnt, 0, 16, s) != cudaSuccess)
            return launched("unwrap workspace reset");
        k_uw_init<T><<<pg, pb, 0, s>>>(phi, F, d.seed, rel, word, bw, be);
        // rounds 0 and 1 over the pixel grid; round 1 also lists the edges
        // that cross components and the roots that stay
        for (int r = 0; r < std::min(rounds, 2); ++r) {
            k_uw_minw<<<pg, pb, 0, s>>>(F, rel, word, bw, flags, r, r == 1 ? el[0] : nullptr, ecnt);
            k_uw_mine<<<pg, pb, 0, s>>>(F, rel, word, bw, be, flags, r);
            if (r == 0)
                k_uw_anchor<<<(unsigned)A, 1024, 0, s>>>(F, bw, be, fe);
            k_uw_hook<T><<<pg, pb, 0, s>>>(F, phi, word, be, rw, flags, r, r == 1 ? rl[0] : nullptr, rcnt);
            k_uw_jump<<<pg, pb, 0, s>>>(F, word, rw, flags, r, status);
            k_uw_flatten<<<pg, pb, 0, s>>>(F, word, rw, bw, be, flags, r);
        }
        // rounds >= 2 on the lists, in and out alternating (round 2 reads
        // the lists round 1 wrote into slot 0)
        for (int r = 2; r < rounds; ++r) {
            const int in = r & 1 ? 1 : 0, out = in ^ 1;
            if (cudaMemsetAsync(ecnt + out, 0, 4, s) != cudaSuccess ||
                cudaMemsetAsync(rcnt + out, 0, 4, s) != cudaSuccess)
                return launched("unwrap list reset");
            k_ul_edges_w<<<UL_GRID, UL_BLOCK, 0, s>>>(rel, word, bw, el[in], ecnt + in, el[out], ecnt + out, d.nx,
                                                      flags, r, status);
            k_ul_edges_e<<<UL_GRID, UL_BLOCK, 0, s>>>(rel, word, bw, be, el[out], ecnt + out, d.nx, flags, r,
                                                      status);
            k_ul_hook<T><<<UL_GRID, UL_BLOCK, 0, s>>>(F, phi, word, be, rw, rl[in], rcnt + in, rl[out], rcnt + out,
                                                      flags, r, status);
            k_ul_jump<<<UL_GRID, UL_BLOCK, 0, s>>>(rw, rl[in], rcnt + in, flags, r, status);
            k_ul_update<<<UL_GRID, UL_BLOCK, 0, s>>>(word, rw, bw, be, rl[in], rcnt + in, flags, r);
        }
        k_uw_finish<T><<<pg, pb, 0, s>>>(F, phi, word, fe, status);
    }
    double *remove = nullptr;
    if (d.align) {
        unsigned long long *minkey = (unsigned long long *)(ws + L.minkey);
        uint32_t *nan_seen = (uint32_t *)(ws + L.nan);
        if (cudaMemsetAsync(minkey, 0xff, 8, s) != cudaSuccess)
            return launched("align workspace reset");
        k_phase_min<T><<<eg, 256, 0, s>>>(phi, N, minkey, nan_seen);
        remove = (double *)(ws + L.remove);
        k_align<T><<<1, 256, 0, s>>>(phi, A, d.ny, d.nx, three_d ? 1 : 0, minkey, nan_seen,
                                     (double *)(ws + L.steps), remove);
    }
    const dim3 cg((unsigned)std::min<long long>((P + 255) / 256, 64), (unsigned)A);
    k_compose<T><<<cg, 256, 0, s>>>(phi, remove, P, N, rytov ? 1 : 0, u0arr, u0s, outc, outr);
    return launched("sinogram preparation");
}

int launches_of(const odt_sino_desc &d)
{
    if (d.kind == ODT_SINO_ALIGN)
        return 3;  // min, align, compose
    int n = (d.kind == ODT_SINO_UNWRAP ? 1 : 2) + (d.align ? 2 : 0);  // (phase,) compose (+ min, align)
    if (d.ny > 0)
        n += 3 + 5 * num_rounds((long long)d.ny * d.nx);  // init, anchor, rounds, finish
    else
        n += 1;
    return n;
}

}  // namespace
}  // namespace odt

using namespace odt;

extern "C" {

odt_status odt_sino_workspace_size(const odt_sino_desc *desc, size_t *bytes)
{
    const odt_status st = check_desc(desc);
    if (st != ODT_OK)
        return st;
    if (!bytes)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL output pointer");
    *bytes = layout_of(*desc).total;
    return ODT_OK;
}

odt_status odt_sino_launch_count(const odt_sino_desc *desc, int32_t *count)
{
    const odt_status st = check_desc(desc);
    if (st != ODT_OK)
        return st;
    if (!count)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL output pointer");
    *count = launches_of(*desc);
    return ODT_OK;
}

odt_status odt_sino_prepare(const odt_sino_desc *desc, const void *sino, void *out, void *workspace,
                            size_t workspace_bytes, void *stream)
{
    const odt_status st = check_desc(desc);
    if (st != ODT_OK)
        return st;
    if (!sino || !out || !workspace)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if (workspace_bytes < layout_of(*desc).total)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "workspace too small");
    const bool dbl = desc->dtype == ODT_DATA_C128 || desc->dtype == ODT_DATA_F64;
    const size_t real_al = dbl ? 8 : 4, cplx_al = 2 * real_al;
    const size_t in_al = (desc->kind == ODT_SINO_ALIGN || desc->kind == ODT_SINO_UNWRAP) ? real_al : cplx_al;
    const size_t out_al = desc->kind == ODT_SINO_RYTOV ? cplx_al : real_al;
    if ((uintptr_t)sino % in_al || (uintptr_t)out % out_al || (desc->u0 && (uintptr_t)desc->u0 % cplx_al) ||
        (uintptr_t)workspace % 256)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "misaligned pointer");
    cudaStream_t s = (cudaStream_t)stream;
    if (dbl)
        return run<double>(*desc, sino, out, (char *)workspace, s);
    return run<float>(*desc, sino, out, (char *)workspace, s);
}

odt_status odt_sino_read_status(const void *workspace, void *stream)
{
    if (!workspace)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL workspace");
    uint32_t v = 0;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess ||
        cudaMemcpy(&v, workspace, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return launched("sinogram status read");
    if (v & STATUS_JUMP)
        return (odt_status)set_error(ODT_ERR_DEVICE_CHECK, "phase unwrap: pointer jumping exceeded its step limit");
    if (v & STATUS_SPLIT)
        return (odt_status)set_error(ODT_ERR_DEVICE_CHECK, "phase unwrap: a frame did not join into one tree");
    return ODT_OK;
}

}  // extern "C"
