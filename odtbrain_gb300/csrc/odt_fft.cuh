// Line transforms shared by the filter stages of the 3D backpropagation.
//
// A "line" is one 1D complex transform (one padded sinogram row, one
// spectrum column, one propagated row).  A group of TPL threads owns a line;
// thread j of the group holds the elements at positions j + r*TPL
// (r < SLOTS) in registers, both before and after the transform, so stage
// kernels can fuse loads, pointwise filters and cropped stores around it.
//
// Pow2Line<N>: radix-8 Stockham autosort FFT (Govindaraju et al., "High
//   performance discrete Fourier transforms on graphics processors", SC'08),
//   with a final radix-4 or radix-2 pass for N = 8^a * {2, 4}.  Passes
//   exchange through two shared-memory buffers used alternately, so each
//   exchange needs a single barrier.
// GenericLine: O(N^2) direct DFT for the sizes that are not powers of two
//   (only reachable with padding=(False, False)); N <= 1024.
//
// Sign convention: DIR = -1 is the forward transform exp(-2 pi i n k / N),
// DIR = +1 the unnormalised backward transform, like FFTW's execute().
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace odt {

// Complex add / subtract as one packed FP32 instruction each (sm_100+
// .f32x2 forms; every component rounds exactly like the scalar operation).
__device__ __forceinline__ unsigned long long f2bits(float2 a) { return *reinterpret_cast<unsigned long long *>(&a); }
__device__ __forceinline__ float2 bitsf2(unsigned long long d) { return *reinterpret_cast<float2 *>(&d); }
__device__ __forceinline__ float2 operator+(float2 a, float2 b)
{
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bitsf2(d);
}
__device__ __forceinline__ float2 operator-(float2 a, float2 b)
{
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bitsf2(d);
}
// s * a + c with a real scalar s (one packed FMA)
__device__ __forceinline__ float2 sfma2(float s, float2 a, float2 c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2bits(make_float2(s, s))), "l"(f2bits(a)), "l"(f2bits(c)));
    return bitsf2(d);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c)  // a*b + c
{
    return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
template <int DIR>
__device__ __forceinline__ float2 mul_i(float2 a)  // a * (DIR * i)
{
    return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
// tw holds exp(-2 pi i m / N); the backward transform uses its conjugate.
template <int DIR>
__device__ __forceinline__ float2 twid(const float2 *tw, int m)
{
    float2 t = tw[m];
    return DIR > 0 ? make_float2(t.x, -t.y) : t;
}

template <int DIR>
__device__ __forceinline__ void dft2(float2 &a, float2 &b)
{
    float2 t = a;
    a = t + b;
    b = t - b;
}

// a + DIR*i*d and a - DIR*i*d
template <int DIR>
__device__ __forceinline__ void add_sub_i(float2 a, float2 d, float2 &p, float2 &m)
{
    p = make_float2(a.x - DIR * d.y, a.y + DIR * d.x);
    m = make_float2(a.x + DIR * d.y, a.y - DIR * d.x);
}

template <int DIR>
__device__ __forceinline__ void dft4(float2 &x0, float2 &x1, float2 &x2, float2 &x3)
{
    const float2 a0 = x0 + x2, a1 = x0 - x2, a2 = x1 + x3, d = x1 - x3;
    x0 = a0 + a2;
    x2 = a0 - a2;
    add_sub_i<DIR>(a1, d, x1, x3);
}

template <int DIR>
__device__ __forceinline__ void dft8(float2 *x)
{
    float2 e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
    float2 o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
    dft4<DIR>(e0, e1, e2, e3);
    dft4<DIR>(o0, o1, o2, o3);
    const float r = 0.70710678118654752440f;
    // o1 *= (1 + DIR i)/sqrt2 ; o2 *= DIR i ; o3 *= (-1 + DIR i)/sqrt2, the
    // 1/sqrt2 folded into packed FMAs with the even half
    const float2 t1 = make_float2(o1.x - DIR * o1.y, o1.y + DIR * o1.x);
    const float2 t3 = make_float2(o3.x + DIR * o3.y, o3.y - DIR * o3.x);  // -o3 rotated
    x[0] = e0 + o0;
    x[4] = e0 - o0;
    x[1] = sfma2(r, t1, e1);
    x[5] = sfma2(-r, t1, e1);
    add_sub_i<DIR>(e2, o2, x[2], x[6]);
    x[3] = sfma2(-r, t3, e3);
    x[7] = sfma2(r, t3, e3);
}

constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

// Barrier over `nthreads` threads (a multiple of 32, whole warps) on named
// barrier `id` (1..15; 0 is __syncthreads'), with shared-memory ordering.
__device__ __forceinline__ void line_sync(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
}

// Exchange-buffer slot of line position p.  The Stockham passes read
// positions j + r*TPL and write positions 8*j' + r (first pass) or
// blocks + 8*r (later passes).
// Row layout (element stride 1, the threads of a half-warp on one line):
//   bits 3..6 XORed into bits 0..3, conflict-free for every pattern.
// Column layout (KX interleaved lines, a half-warp spans 8 lines and 2
//   positions): one slot of padding after every 8 positions, conflict-free
//   there, and every slot is a per-thread base plus a compile-time offset,
//   so those exchanges need no index arithmetic per element.
template <bool PAD>
__device__ __forceinline__ int xslot(int p)
{
    return PAD ? p + (p >> 3) : p ^ ((p >> 3) & 15);
}
// Slots a line of n positions occupies in an exchange buffer of the layout.
template <bool PAD>
__host__ __device__ constexpr int xslots(int n)
{
    return PAD ? n + n / 8 + 1 : n;
}
constexpr int ipow8(int k) { return k == 0 ? 1 : 8 * ipow8(k - 1); }

// Shared-memory twiddle region of a line: the plain table exp(-2 pi i m / N)
// (N entries), then for power-of-two lines the twiddles of the second
// radix-8 pass (Ns = 8) stored contiguously per thread class jm: entry
// jm*7 + r-1 = exp(-2 pi i r jm / 64), the plain table's entry r*jm*N/64.
// Read from the plain table, the 8 distinct twiddles a warp needs in that
// pass lie on one or two banks (4- to 8-way conflicts); read from this
// table they lie on distinct banks.
constexpr int TW_P1 = 56;
__host__ __device__ constexpr int tw_slots(int n) { return n + TW_P1; }
// Optional third table, for lines whose third radix-8 pass (Ns = 64) reads
// its twiddles per thread class jm = j mod 64: entry jm*7 + r-1 =
// exp(-2 pi i r jm / 512), the plain table's entry r*jm*N/512.  Read from
// it, a warp's twiddles lie on distinct banks at a per-thread base plus a
// constant offset (from the plain table the even r read with 2- and 4-way
// conflicts, at addresses computed per r).
constexpr int TW_P2 = 64 * 7;
__host__ __device__ constexpr int tw_slots2(int n) { return n + TW_P1 + TW_P2; }

// Power-of-two line, 64 <= N <= 4096.
template <int N_>
struct Pow2Line {
    static constexpr int N = N_;
    static constexpr int TPL = N / 8;
    static constexpr int SLOTS = 8;
    static constexpr int P8 = ilog2c(N) / 3;
    static constexpr int TAIL = N / ipow8(P8);  // 1, 2 or 4
    int n;  // == N, kept for a uniform interface with GenericLine
    __device__ __forceinline__ int size() const { return N; }

    // v: positions j + r*TPL in, same positions out.  `line[0/1]` point at
    // element 0 of this line in the two exchange buffers; `es` is the
    // element stride.  `flip` alternates the buffers across exchanges.
    // PAD selects the exchange layout (xslot): false for rows, true for
    // interleaved columns.
    // bar > 0: the line's TPL threads are consecutive warps and sync on
    // named barrier `bar` (only they share the line's buffers); 0: the whole
    // CTA syncs.
    // TW2: the twiddle region also holds the third table (tw_slots2).
    template <int DIR, bool PAD = false, bool TW2 = false>
    __device__ __forceinline__ void run(float2 (&v)[8], int j, float2 *line0, float2 *line1, int es,
                                        const float2 *tw, int &flip, int bar = 0) const
    {
        int Ns = 1;
#pragma unroll
        for (int pass = 0; pass < P8; ++pass) {
            if (pass == 1) {
                const float2 *t1 = tw + N + (j & 7) * 7;
#pragma unroll
                for (int r = 1; r < 8; ++r)
                    v[r] = cmul(v[r], twid<DIR>(t1, r - 1));
            } else if (pass == 2 && TW2) {
                const float2 *t2 = tw + N + TW_P1 + (j & 63) * 7;
#pragma unroll
                for (int r = 1; r < 8; ++r)
                    v[r] = cmul(v[r], twid<DIR>(t2, r - 1));
            } else if (pass > 1) {
                const int jm = j & (Ns - 1);
                const int stp = jm * (N / (Ns * 8));
#pragma unroll
                for (int r = 1; r < 8; ++r)
                    v[r] = cmul(v[r], twid<DIR>(tw, r * stp));
            }
            dft8<DIR>(v);
            if (pass == P8 - 1 && TAIL == 1)
                break;
            float2 *b = flip ? line1 : line0;
            flip ^= 1;
            const int idxD = (j / Ns) * Ns * 8 + (j & (Ns - 1));
#pragma unroll
            for (int r = 0; r < 8; ++r)
                b[xslot<PAD>(idxD + r * Ns) * es] = v[r];
            if (bar > 0)
                line_sync(bar, TPL);
            else
                __syncthreads();
#pragma unroll
            for (int r = 0; r < 8; ++r)
                v[r] = b[xslot<PAD>(j + r * TPL) * es];
            Ns *= 8;
        }
        if (TAIL == 4) {
#pragma unroll
            for (int g = 0; g < 2; ++g) {
                const int jj = j + g * TPL;
                float2 x0 = v[g], x1 = v[g + 2], x2 = v[g + 4], x3 = v[g + 6];
                x1 = cmul(x1, twid<DIR>(tw, jj));
                x2 = cmul(x2, twid<DIR>(tw, 2 * jj));
                x3 = cmul(x3, twid<DIR>(tw, 3 * jj));
                dft4<DIR>(x0, x1, x2, x3);
                v[g] = x0;
                v[g + 2] = x1;
                v[g + 4] = x2;
                v[g + 6] = x3;
            }
        } else if (TAIL == 2) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int jj = j + q * TPL;
                float2 b = cmul(v[q + 4], twid<DIR>(tw, jj));
                float2 a = v[q];
                v[q] = a + b;
                v[q + 4] = a - b;
            }
        }
    }
};

// Any N <= TPL*SLOTS: direct DFT through shared memory (unpadded slots).
struct GenericLine {
    static constexpr int TPL = 64;
    static constexpr int SLOTS = 16;
    int n;
    __device__ __forceinline__ int size() const { return n; }

    // (TW2 is accepted for a uniform interface; the direct DFT has no passes)
    template <int DIR, bool PAD = false, bool TW2 = false>
    __device__ __forceinline__ void run(float2 (&v)[16], int j, float2 *line0, float2 *line1, int es,
                                        const float2 *tw, int &flip, int bar = 0) const
    {
        float2 *b = flip ? line1 : line0;
        flip ^= 1;
#pragma unroll
        for (int r = 0; r < SLOTS; ++r) {
            const int k = j + r * TPL;
            if (k < n)
                b[k * es] = v[r];
        }
        __syncthreads();
#pragma unroll 1
        for (int r = 0; r < SLOTS; ++r) {
            const int k = j + r * TPL;
            if (k >= n)
                break;
            float2 acc = make_float2(0.f, 0.f);
            int m = 0;
            for (int i = 0; i < n; ++i) {
                acc = cfma(b[i * es], twid<DIR>(tw, m), acc);
                m += k;
                if (m >= n)
                    m -= n;
            }
            v[r] = acc;
        }
    }
};

}  // namespace odt
