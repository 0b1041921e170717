// Learned filter gain: a 4-layer MLP on the tensor cores.
//
// For every angle a and padded frequency k = (ky, kx) the network maps the
// features (2*kx/lNx, 2*ky/lNy in fftfreq order, an angle feature, an
// angular-gap feature) to a complex gain  gamma = 1 + out_re + i*out_im
// that multiplies the filter of that angle (the angle_gain argument of
// odt_bpp3d_execute_gain).  Layers: 4 -> 64 -> 64 -> 64 -> 2 with SiLU
// activations, BF16 operands and FP32 accumulation on the tensor cores
// (mma.sync.m16n8k16 with BF16 inputs).  The input width is padded to 16 and
// the output width to 8 so that every layer is a tensor-core product; the
// padding columns of W1 and rows of W4 are zero.
//
// Fragment layout of mma.m16n8k16 (per warp, lane = 4*g + t):
//   A (16x16, row-major)   a0a1=(g, 2t..2t+1) a2a3=(g+8, 2t..) a4a5=(g, 2t+8..)
//                          a6a7=(g+8, 2t+8..)
//   B (16x8, column-major) b0b1=(2t..2t+1, g) b2b3=(2t+8.., g)
//   C/D (16x8, FP32)       c0c1=(g, 2t..2t+1) c2c3=(g+8, 2t..)
// so the accumulators of two adjacent 8-column tiles are exactly the A
// operand of the next layer's 16-column k-tile: a warp carries 16 points
// through all layers in registers.
//
// The points evaluated are, per angle, either every padded spectrum position
// or a caller's list of positions (the filter's support: elsewhere the
// filter is zero and the gain has no effect).
//
// Training: k_mlp_backward_data recomputes the forward for 16 points per
// warp, back-propagates the gain gradient through the layers (with the
// transposed weights, again on the tensor cores) and stores the BF16
// activations and pre-activation gradients; k_mlp_wgrad forms every weight
// and bias gradient as a split-K product over the points (a column of ones
// gives the bias) and adds its partial sums with atomics.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/odtbrain_gb300.h"
#include "mlp_tc.cuh"
#include "odt_fft.cuh"
#include "odt_internal.cuh"

namespace odt {
namespace {

constexpr int MLP_IN = 16;    // padded input width (4 features)
constexpr int MLP_H = 64;     // hidden width
constexpr int MLP_OUT = 8;    // padded output width (2 outputs)
constexpr int MLP_OUTP = 16;  // output gradient padded to one k-tile
// shared-memory row strides (BF16 elements) of the weight matrices: 8
// elements of padding make the B-fragment loads of a warp conflict-free
constexpr int LD16 = MLP_IN + 8;
constexpr int LD64 = MLP_H + 8;

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ uint32_t pair_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    __nv_bfloat162 v;
    v.x = lo;
    v.y = hi;
    return *reinterpret_cast<uint32_t *>(&v);
}

// fast reciprocal: the activations are rounded to BF16 next (C5 gain
// inference: 0.37 -> 0.18 ms with the IEEE division replaced)
__device__ __forceinline__ float sigmoid(float z) { return __fdividef(1.f, 1.f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid(z); }
__device__ __forceinline__ float silu_grad(float z)
{
    const float s = sigmoid(z);
    return s * (1.f + z * (1.f - s));
}

// B fragment of a K x N operand whose column n is row n of `rows` (row
// stride ld), at k-tile kt and n-tile nt.
__device__ __forceinline__ void load_b(const __nv_bfloat16 *rows, int ld, int kt, int nt, int lane, uint32_t &b0,
                                       uint32_t &b1)
{
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16 *row = rows + (nt * 8 + g) * ld + kt * 16 + 2 * t;
    b0 = *reinterpret_cast<const uint32_t *>(row);
    b1 = *reinterpret_cast<const uint32_t *>(row + 8);
}

// Accumulators of n-tiles (2kt, 2kt+1) -> A fragment of k-tile kt.
__device__ __forceinline__ void acc_to_a(const float (&d0)[4], const float (&d1)[4], uint32_t (&a)[4])
{
    a[0] = pack_bf16(d0[0], d0[1]);
    a[1] = pack_bf16(d0[2], d0[3]);
    a[2] = pack_bf16(d1[0], d1[1]);
    a[3] = pack_bf16(d1[2], d1[3]);
}

struct MlpWeights {
    const __nv_bfloat16 *w1, *w2, *w3, *w4;  // [out][in]: 64x16, 64x64, 64x64, 8x64
    const __nv_bfloat16 *w2t, *w3t, *w4t;    // [in][out]: 64x64, 64x64, 64x16
    const float *b1, *b2, *b3, *b4;          // 64, 64, 64, 8
};

struct SmemForward {
    __nv_bfloat16 w1[MLP_H * LD16];
    __nv_bfloat16 w2[MLP_H * LD64];
    __nv_bfloat16 w3[MLP_H * LD64];
    __nv_bfloat16 w4[MLP_OUT * LD64];
    float b1[MLP_H], b2[MLP_H], b3[MLP_H], b4[MLP_OUT];
};

struct SmemBackward {
    SmemForward f;
    __nv_bfloat16 w2t[MLP_H * LD64];
    __nv_bfloat16 w3t[MLP_H * LD64];
    __nv_bfloat16 w4t[MLP_H * LD16];
};

// Copy a rows x K BF16 matrix into shared rows of stride ld.
__device__ void copy_rows(__nv_bfloat16 *dst, const __nv_bfloat16 *src, int rows, int K, int ld)
{
    const int words = rows * K / 2;
    for (int i = threadIdx.x; i < words; i += blockDim.x) {
        const int r = i / (K / 2), c = i % (K / 2);
        reinterpret_cast<uint32_t *>(dst + r * ld)[c] = reinterpret_cast<const uint32_t *>(src)[i];
    }
}

__device__ void load_forward(const MlpWeights &W, SmemForward &S)
{
    copy_rows(S.w1, W.w1, MLP_H, MLP_IN, LD16);
    copy_rows(S.w2, W.w2, MLP_H, MLP_H, LD64);
    copy_rows(S.w3, W.w3, MLP_H, MLP_H, LD64);
    copy_rows(S.w4, W.w4, MLP_OUT, MLP_H, LD64);
    for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
        S.b1[i] = W.b1[i];
        S.b2[i] = W.b2[i];
        S.b3[i] = W.b3[i];
    }
    if (threadIdx.x < MLP_OUT)
        S.b4[threadIdx.x] = W.b4[threadIdx.x];
}

struct MlpGrid {
    int A, lNy, lNx;
    const int *pos;            // spectrum positions ky*lNx + kx evaluated
                               // (NULL: all lNy*lNx)
    int npos;                  // positions per angle
    long long P;               // A * npos points
    const float2 *angle_feat;  // per angle: (angle feature, gap feature)
};

// Spectrum position of the j-th evaluated point of an angle; positions
// outside [0, lNy*lNx) in a caller's list give -1 (the point is skipped).
__device__ __forceinline__ int position(const MlpGrid &Gd, int j)
{
    const int k = Gd.pos ? __ldg(Gd.pos + j) : j;
    return (unsigned)k < (unsigned)(Gd.lNy * Gd.lNx) ? k : -1;
}

// Point p = a*npos + j stands for the gain entry a*lNy*lNx + pos[j] (-1:
// skipped).
__device__ __forceinline__ long long gain_index(const MlpGrid &Gd, long long p)
{
    const int a = (int)(p / Gd.npos);
    const int k = position(Gd, (int)(p - (long long)a * Gd.npos));
    return k < 0 ? -1 : (long long)a * Gd.lNy * Gd.lNx + k;
}

// Features of point p.
__device__ __forceinline__ void point_features(const MlpGrid &Gd, long long p, float (&f)[4])
{
    const int a = (int)(p / Gd.npos);
    const int k = max(position(Gd, (int)(p - (long long)a * Gd.npos)), 0);
    const int ky = k / Gd.lNx, kx = k - ky * Gd.lNx;
    // fftfreq order: index m stands for m (m <= (N-1)/2) or m - N
    const int hx = (Gd.lNx - 1) / 2, hy = (Gd.lNy - 1) / 2;
    f[0] = 2.f * (float)(kx <= hx ? kx : kx - Gd.lNx) / (float)Gd.lNx;
    f[1] = 2.f * (float)(ky <= hy ? ky : ky - Gd.lNy) / (float)Gd.lNy;
    const float2 af = Gd.angle_feat[a];
    f[2] = af.x;
    f[3] = af.y;
}

// Input A fragment of 16 points starting at p0 (features in columns 0..3).
__device__ __forceinline__ void input_fragment(const MlpGrid &Gd, long long p0, int lane, uint32_t (&a)[4],
                                               float (&feat)[2][4])
{
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const long long idx = p0 + g + 8 * h;
        if (idx < Gd.P) {
            point_features(Gd, idx, feat[h]);
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c)
                feat[h][c] = 0.f;
        }
    }
    a[0] = a[1] = a[2] = a[3] = 0u;
    if (t == 0) {
        a[0] = pack_bf16(feat[0][0], feat[0][1]);
        a[1] = pack_bf16(feat[1][0], feat[1][1]);
    } else if (t == 1) {
        a[0] = pack_bf16(feat[0][2], feat[0][3]);
        a[1] = pack_bf16(feat[1][2], feat[1][3]);
    }
}

// One dense layer on 16 points: D[nt] = bias + sum_kt A[kt] * B[kt][nt].
template <int KT, int NT>
__device__ __forceinline__ void dense(const uint32_t (&A)[KT][4], const __nv_bfloat16 *rows, int ld,
                                      const float *bias, int lane, float (&D)[NT][4])
{
    const int t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const float bx = bias ? bias[nt * 8 + 2 * t] : 0.f;
        const float by = bias ? bias[nt * 8 + 2 * t + 1] : 0.f;
        D[nt][0] = bx;
        D[nt][1] = by;
        D[nt][2] = bx;
        D[nt][3] = by;
#pragma unroll
        for (int kt = 0; kt < KT; ++kt) {
            uint32_t b0, b1;
            load_b(rows, ld, kt, nt, lane, b0, b1);
            mma_bf16(D[nt], A[kt], b0, b1);
        }
    }
}

template <int NT>
__device__ __forceinline__ void silu_of(const float (&Z)[NT][4], float (&H)[NT][4])
{
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            H[nt][i] = silu(Z[nt][i]);
}

template <int NT>
__device__ __forceinline__ void to_a(const float (&H)[NT][4], uint32_t (&A)[NT / 2][4])
{
#pragma unroll
    for (int kt = 0; kt < NT / 2; ++kt)
        acc_to_a(H[2 * kt], H[2 * kt + 1], A[kt]);
}

// ---------------------------------------------------------------------------
// Inference: gamma for every (angle, frequency) point.  Persistent: every
// warp walks 16-point groups with a grid stride, the weights stay in shared
// memory.
constexpr int FWD_WARPS = 8;
// Inference and the data part of the backward pass run on tcgen05
// (k_mlp_forward_tc, k_mlp_backward_data_tc) unless odt_mlp_select_kernels
// picks the same network on the warp-level mma.sync path (k_mlp_forward,
// k_mlp_backward_data), which is kept for comparison.
std::atomic<int> g_mlp_tensor_memory{1};

__global__ void __launch_bounds__(32 * FWD_WARPS) k_mlp_forward(MlpWeights W, MlpGrid Gd, float2 *gain)
{
    __shared__ SmemForward S;
    load_forward(W, S);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const long long groups = (Gd.P + 15) / 16;
    for (long long grp = (long long)blockIdx.x * FWD_WARPS + warp; grp < groups;
         grp += (long long)gridDim.x * FWD_WARPS) {
        const long long p0 = grp * 16;
        uint32_t A0[1][4];
        float feat[2][4];
        input_fragment(Gd, p0, lane, A0[0], feat);
        float Z[8][4], H[8][4], O[1][4];
        uint32_t A[4][4];
        dense<1, 8>(A0, S.w1, LD16, S.b1, lane, Z);
        silu_of<8>(Z, H);
        to_a<8>(H, A);
        dense<4, 8>(A, S.w2, LD64, S.b2, lane, Z);
        silu_of<8>(Z, H);
        to_a<8>(H, A);
        dense<4, 8>(A, S.w3, LD64, S.b3, lane, Z);
        silu_of<8>(Z, H);
        to_a<8>(H, A);
        dense<4, 1>(A, S.w4, LD64, S.b4, lane, O);
        if (t == 0) {
            const long long i0 = p0 + g, i1 = p0 + g + 8;
            const long long k0 = i0 < Gd.P ? gain_index(Gd, i0) : -1;
            const long long k1 = i1 < Gd.P ? gain_index(Gd, i1) : -1;
            if (k0 >= 0)
                gain[k0] = make_float2(1.f + O[0][0], O[0][1]);
            if (k1 >= 0)
                gain[k1] = make_float2(1.f + O[0][2], O[0][3]);
        }
    }
}

// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05.mma, accumulators in
// tensor memory; see mlp_tc.cuh for the operand layout).  Two warp groups per
// CTA, each carrying a tile of 128 points (one per thread and TMEM lane)
// through the four layers; the tiles are walked with a grid stride.
constexpr int TC_SLOTS = 2;
constexpr int TC_THREADS = 128 * TC_SLOTS;
constexpr uint32_t TC_TMEM_COLS = 128;  // 64 FP32 accumulator columns per slot
constexpr uint64_t kTcWaitNs = 1000000000ull;

struct SmemTc {
    uint8_t a[TC_SLOTS][128 * MLP_H * 2];  // per slot: the A operand, 128 x (16 or 64) BF16
    uint8_t w2[MLP_H * MLP_H * 2];         // B operands: the weights [out][in], K-major
    uint8_t w3[MLP_H * MLP_H * 2];
    uint8_t w1[MLP_H * MLP_IN * 2];
    uint8_t w4[16 * MLP_H * 2];            // 16 output rows (2.. zero): N = 16
    float b1[MLP_H], b2[MLP_H], b3[MLP_H], b4[MLP_OUT];
    uint64_t bar[TC_SLOTS];                // MMA completion, one per slot
    uint32_t tmem_base;
    int abort;                             // a wait gave up
};
constexpr size_t TC_SMEM = sizeof(SmemTc) + 1024;  // + alignment of the base

// Status of the tensor-core kernels (bit 0: an MMA completion wait gave
// up), read and cleared by odt_mlp_read_status.
__device__ int g_mlp_status;

// rows x K row-major BF16 -> canonical K-major layout of rows_dst rows (rows
// beyond `rows` zero).
__device__ void tc_copy_kmajor(uint8_t *dst, const __nv_bfloat16 *src, int rows, int rows_dst, int K)
{
    const int kch = K / 8;
    for (int i = threadIdx.x; i < rows_dst * kch; i += blockDim.x) {
        const int r = i / kch, c = i - (i / kch) * kch;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r < rows)
            v = reinterpret_cast<const uint4 *>(src + (size_t)r * K)[c];
        *reinterpret_cast<uint4 *>(dst + tc::kmaj(r, c, kch)) = v;
    }
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_forward_tc(MlpWeights W, MlpGrid Gd, float2 *gain)
{
    extern __shared__ uint8_t tc_smem_raw[];
    SmemTc &S = *reinterpret_cast<SmemTc *>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, slot = tid >> 7, row = tid & 127, warp = tid >> 5;
    tc_copy_kmajor(S.w1, W.w1, MLP_H, MLP_H, MLP_IN);
    tc_copy_kmajor(S.w2, W.w2, MLP_H, MLP_H, MLP_H);
    tc_copy_kmajor(S.w3, W.w3, MLP_H, MLP_H, MLP_H);
    tc_copy_kmajor(S.w4, W.w4, MLP_OUT, 16, MLP_H);
    for (int i = tid; i < MLP_H; i += blockDim.x) {
        S.b1[i] = W.b1[i];
        S.b2[i] = W.b2[i];
        S.b3[i] = W.b3[i];
    }
    if (tid < MLP_OUT)
        S.b4[tid] = W.b4[tid];
    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        S.abort = 0;
        fence_mbar_init();
    }
    if (warp == 0)
        tc::tmem_alloc(&S.tmem_base, TC_TMEM_COLS);
    fence_proxy_async_smem();  // the weight stores, before the MMAs read them
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t d_tmem = S.tmem_base + (uint32_t)slot * 64u;
    const uint32_t lane_addr = d_tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    uint8_t *abuf = S.a[slot];
    const uint32_t a_s = smem_u32(abuf);
    volatile int *abort = &S.abort;
    uint32_t phase = 0;
    const int bar_id = 1 + slot;

    // The group's A operand is in shared memory: one thread issues the
    // layer's K/16 MMAs into the slot's TMEM columns and commits them; the
    // group waits for the products.
    auto layer = [&](const uint8_t *b, int kchunks, uint32_t idesc) {
        fence_proxy_async_smem();  // this thread's operand stores -> async proxy
        tc::fence_before_sync();   // and its earlier TMEM loads, before the barrier
        line_sync(bar_id, 128);
        if (row == 0) {
            tc::fence_after_sync();
            const uint32_t sbo = 128u * kchunks, b_s = smem_u32(b);
            for (int k = 0; k < kchunks / 2; ++k)
                tc::mma(d_tmem, tc::smem_desc(a_s + 256u * k, 128u, sbo), tc::smem_desc(b_s + 256u * k, 128u, sbo),
                        idesc, k > 0 ? 1u : 0u);
            tc::commit(&S.bar[slot]);
        }
        const bool ok = !*abort && mbar_wait(&S.bar[slot], phase, kTcWaitNs);
        phase ^= 1u;
        if (!ok)
            *abort = 1;
        tc::fence_after_sync();
    };
    // bias + SiLU of the 64 accumulator columns -> BF16 A operand row
    auto hidden = [&](const float *bias) {
        uint32_t r[4][16];
#pragma unroll
        for (int c = 0; c < 4; ++c)
            tc::tmem_ld16(lane_addr + 16u * c, r[c]);
#pragma unroll
        for (int c = 0; c < 4; ++c)
            tc::tmem_wait(r[c]);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            float z[8];
#pragma unroll
            for (int i = 0; i < 8; ++i)
                z[i] = silu(__uint_as_float(r[c >> 1][(c & 1) * 8 + i]) + bias[8 * c + i]);
            *reinterpret_cast<uint4 *>(abuf + tc::kmaj(row, c, 8)) =
                make_uint4(pack_bf16(z[0], z[1]), pack_bf16(z[2], z[3]), pack_bf16(z[4], z[5]),
                           pack_bf16(z[6], z[7]));
        }
    };

    const long long ntiles = (Gd.P + 127) / 128;
    for (long long t = (long long)blockIdx.x * TC_SLOTS + slot; t < ntiles; t += (long long)gridDim.x * TC_SLOTS) {
        const long long p = t * 128 + row;
        float f[4] = {0.f, 0.f, 0.f, 0.f};
        if (p < Gd.P)
            point_features(Gd, p, f);
        // A0 = (f0 .. f3, 0 ..) of width 16: two 16-byte chunks
        *reinterpret_cast<uint4 *>(abuf + tc::kmaj(row, 0, 2)) =
            make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), 0u, 0u);
        *reinterpret_cast<uint4 *>(abuf + tc::kmaj(row, 1, 2)) = make_uint4(0u, 0u, 0u, 0u);
        layer(S.w1, MLP_IN / 8, tc::idesc_bf16(128, 64));
        hidden(S.b1);
        layer(S.w2, MLP_H / 8, tc::idesc_bf16(128, 64));
        hidden(S.b2);
        layer(S.w3, MLP_H / 8, tc::idesc_bf16(128, 64));
        hidden(S.b3);
        layer(S.w4, MLP_H / 8, tc::idesc_bf16(128, 16));
        uint32_t r[16];
        tc::tmem_ld16(lane_addr, r);
        tc::tmem_wait(r);
        if (p < Gd.P) {
            const long long k = gain_index(Gd, p);
            if (k >= 0)
                gain[k] = make_float2(1.f + (__uint_as_float(r[0]) + S.b4[0]), __uint_as_float(r[1]) + S.b4[1]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (*abort) {
        // a wait gave up: report it, and give the MMAs still in flight a
        // last bounded wait before the accumulators are released
        if (row == 0)
            mbar_wait(&S.bar[slot], phase ^ 1u, kTcWaitNs);
        if (tid == 0)
            atomicOr(&g_mlp_status, 1);
        __syncthreads();
    }
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(S.tmem_base, TC_TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------
// Backward, data part: stores per point the BF16 layer inputs H0 (16 wide),
// H1..H3 (64) and pre-activation gradients DZ1..DZ3 (64), DZ4 (16: d out_re,
// d out_im, zeros).
struct MlpStore {
    __nv_bfloat16 *h0, *h1, *h2, *h3;
    __nv_bfloat16 *dz1, *dz2, *dz3, *dz4;
};

// Store 16 x (8*NT) FP32 values as BF16 rows of width 8*NT.
template <int NT>
__device__ __forceinline__ void store_rows(__nv_bfloat16 *dst, long long p0, long long P, int lane,
                                           const float (&D)[NT][4])
{
    const int g = lane >> 2, t = lane & 3;
    constexpr int w = NT * 8;
    const long long i0 = p0 + g, i1 = p0 + g + 8;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        if (i0 < P)
            *reinterpret_cast<uint32_t *>(dst + i0 * w + nt * 8 + 2 * t) = pack_bf16(D[nt][0], D[nt][1]);
        if (i1 < P)
            *reinterpret_cast<uint32_t *>(dst + i1 * w + nt * 8 + 2 * t) = pack_bf16(D[nt][2], D[nt][3]);
    }
}

template <int NT>
__device__ __forceinline__ void times_silu_grad(float (&D)[NT][4], const float (&Z)[NT][4])
{
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            D[nt][i] *= silu_grad(Z[nt][i]);
}

constexpr int BWD_WARPS = 4;

__global__ void __launch_bounds__(32 * BWD_WARPS) k_mlp_backward_data(MlpWeights W, MlpGrid Gd,
                                                                      const float2 *dgain, MlpStore St)
{
    __shared__ SmemBackward S;
    load_forward(W, S.f);
    copy_rows(S.w2t, W.w2t, MLP_H, MLP_H, LD64);
    copy_rows(S.w3t, W.w3t, MLP_H, MLP_H, LD64);
    copy_rows(S.w4t, W.w4t, MLP_H, MLP_OUTP, LD16);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const long long P = Gd.P;
    const long long groups = (P + 15) / 16;
    for (long long grp = (long long)blockIdx.x * BWD_WARPS + warp; grp < groups;
         grp += (long long)gridDim.x * BWD_WARPS) {
        const long long p0 = grp * 16;
        uint32_t A0[1][4];
        float feat[2][4];
        input_fragment(Gd, p0, lane, A0[0], feat);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const long long idx = p0 + g + 8 * h;
            if (idx < P) {
                // lane t writes columns 4t..4t+3; the features are columns 0..3
                uint2 v;
                v.x = t == 0 ? pack_bf16(feat[h][0], feat[h][1]) : 0u;
                v.y = t == 0 ? pack_bf16(feat[h][2], feat[h][3]) : 0u;
                *reinterpret_cast<uint2 *>(St.h0 + idx * MLP_IN + 4 * t) = v;
            }
        }
        float Z1[8][4], Z2[8][4], Z3[8][4], T[8][4];
        uint32_t A[4][4];
        dense<1, 8>(A0, S.f.w1, LD16, S.f.b1, lane, Z1);
        silu_of<8>(Z1, T);
        store_rows<8>(St.h1, p0, P, lane, T);
        to_a<8>(T, A);
        dense<4, 8>(A, S.f.w2, LD64, S.f.b2, lane, Z2);
        silu_of<8>(Z2, T);
        store_rows<8>(St.h2, p0, P, lane, T);
        to_a<8>(T, A);
        dense<4, 8>(A, S.f.w3, LD64, S.f.b3, lane, Z3);
        silu_of<8>(Z3, T);
        store_rows<8>(St.h3, p0, P, lane, T);

        // output gradient (d out_re, d out_im) = (Re, Im) of the gain gradient
        float dO[2][2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const long long idx = p0 + g + 8 * h;
            const long long gi = idx < P ? gain_index(Gd, idx) : -1;
            const float2 d = gi >= 0 ? dgain[gi] : make_float2(0.f, 0.f);
            dO[h][0] = d.x;
            dO[h][1] = d.y;
            if (idx < P) {
                uint2 v;
                v.x = t == 0 ? pack_bf16(d.x, d.y) : 0u;
                v.y = 0u;
                *reinterpret_cast<uint2 *>(St.dz4 + idx * MLP_OUTP + 4 * t) = v;
            }
        }
        uint32_t Ad[1][4] = {{0u, 0u, 0u, 0u}};
        if (t == 0) {
            Ad[0][0] = pack_bf16(dO[0][0], dO[0][1]);
            Ad[0][1] = pack_bf16(dO[1][0], dO[1][1]);
        }
        // dh3 = dout W4, then through the SiLU of layer 3
        dense<1, 8>(Ad, S.w4t, LD16, nullptr, lane, T);
        times_silu_grad<8>(T, Z3);
        store_rows<8>(St.dz3, p0, P, lane, T);
        to_a<8>(T, A);
        dense<4, 8>(A, S.w3t, LD64, nullptr, lane, T);  // dh2 = dz3 W3
        times_silu_grad<8>(T, Z2);
        store_rows<8>(St.dz2, p0, P, lane, T);
        to_a<8>(T, A);
        dense<4, 8>(A, S.w2t, LD64, nullptr, lane, T);  // dh1 = dz2 W2
        times_silu_grad<8>(T, Z1);
        store_rows<8>(St.dz1, p0, P, lane, T);
    }
}

// ---------------------------------------------------------------------------
// Backward, data part, on tcgen05: one warp group (128 threads) per CTA
// carries a tile of 128 points (thread = point = TMEM lane).  The forward is
// recomputed with the pre-activations Z1, Z2, Z3 left in TMEM columns
// [0, 64), [64, 128), [128, 192); the back-propagated products dH3, dH2,
// dH1 (dZ times the transposed weights) land in columns [192, 256).  Every
// layer input and pre-activation gradient is stored in BF16 (MlpStore) for
// the weight-gradient kernels, exactly as k_mlp_backward_data stores them.
constexpr uint32_t TB_TMEM_COLS = 256;

struct SmemTb {
    uint8_t a[128 * MLP_H * 2];            // the A operand, 128 x (16 or 64) BF16
    uint8_t w2[MLP_H * MLP_H * 2], w3[MLP_H * MLP_H * 2];    // [out][in]
    uint8_t w2t[MLP_H * MLP_H * 2], w3t[MLP_H * MLP_H * 2];  // [in][out]
    uint8_t w1[MLP_H * MLP_IN * 2];        // 64 x 16
    uint8_t w4t[MLP_H * MLP_OUTP * 2];     // 64 x 16 (W4 transposed)
    float b1[MLP_H], b2[MLP_H], b3[MLP_H];
    uint64_t bar;
    uint32_t tmem_base;
    int abort;
};
// at least 100 KB of shared memory, so that no more than two CTAs (the
// 512 TMEM columns of an SM) share an SM: a third would wait in its TMEM
// allocation
constexpr size_t TB_SMEM = sizeof(SmemTb) + 1024 > 100 * 1024 ? sizeof(SmemTb) + 1024 : 100 * 1024;

__device__ __forceinline__ float silu_grad_of(float z)
{
    const float sg = sigmoid(z);
    return sg * (1.f + z * (1.f - sg));
}

__global__ void __launch_bounds__(128, 1) k_mlp_backward_data_tc(MlpWeights W, MlpGrid Gd, const float2 *dgain,
                                                                 MlpStore St)
{
    extern __shared__ uint8_t tb_smem_raw[];
    SmemTb &S = *reinterpret_cast<SmemTb *>((reinterpret_cast<uintptr_t>(tb_smem_raw) + 1023) & ~(uintptr_t)1023);
    const int row = threadIdx.x, warp = row >> 5;
    tc_copy_kmajor(S.w1, W.w1, MLP_H, MLP_H, MLP_IN);
    tc_copy_kmajor(S.w2, W.w2, MLP_H, MLP_H, MLP_H);
    tc_copy_kmajor(S.w3, W.w3, MLP_H, MLP_H, MLP_H);
    tc_copy_kmajor(S.w2t, W.w2t, MLP_H, MLP_H, MLP_H);
    tc_copy_kmajor(S.w3t, W.w3t, MLP_H, MLP_H, MLP_H);
    tc_copy_kmajor(S.w4t, W.w4t, MLP_H, MLP_H, MLP_OUTP);
    for (int i = row; i < MLP_H; i += blockDim.x) {
        S.b1[i] = W.b1[i];
        S.b2[i] = W.b2[i];
        S.b3[i] = W.b3[i];
    }
    if (row == 0) {
        mbar_init(&S.bar, 1);
        S.abort = 0;
        fence_mbar_init();
    }
    if (warp == 0)
        tc::tmem_alloc(&S.tmem_base, TB_TMEM_COLS);
    fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t lane_base = S.tmem_base + ((uint32_t)(32 * warp) << 16);
    const uint32_t a_s = smem_u32(S.a);
    volatile int *abort = &S.abort;
    uint32_t phase = 0;
    // D (TMEM column col0) = A * B: K/16 MMAs issued by thread 0, then the
    // tile waits for them
    auto mma_into = [&](uint32_t col0, const uint8_t *b, int kchunks, int N) {
        fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (row == 0) {
            tc::fence_after_sync();
            const uint32_t sbo = 128u * kchunks, b_s = smem_u32(b);
            for (int k = 0; k < kchunks / 2; ++k)
                tc::mma(S.tmem_base + col0, tc::smem_desc(a_s + 256u * k, 128u, sbo),
                        tc::smem_desc(b_s + 256u * k, 128u, sbo), tc::idesc_bf16(128, N), k > 0 ? 1u : 0u);
            tc::commit(&S.bar);
        }
        const bool ok = !*abort && mbar_wait(&S.bar, phase, kTcWaitNs);
        phase ^= 1u;
        if (!ok)
            *abort = 1;
        tc::fence_after_sync();
    };
    // 64 columns of this thread's lane from column col0
    auto ld64 = [&](uint32_t col0, uint32_t (&r)[4][16]) {
#pragma unroll
        for (int c = 0; c < 4; ++c)
            tc::tmem_ld16(lane_base + col0 + 16u * c, r[c]);
#pragma unroll
        for (int c = 0; c < 4; ++c)
            tc::tmem_wait(r[c]);
    };
    // 8 BF16 values as one 16-byte chunk of the A operand (K = 64) and of
    // the store row
    auto put8 = [&](const float (&v)[8], int c, __nv_bfloat16 *grow) {
        const uint4 q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                                   pack_bf16(v[6], v[7]));
        *reinterpret_cast<uint4 *>(S.a + tc::kmaj(row, c, 8)) = q;
        if (grow)
            reinterpret_cast<uint4 *>(grow)[c] = q;
    };
    const long long P = Gd.P;
    const long long ntiles = (P + 127) / 128;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long p = t * 128 + row;
        const bool valid = p < P;
        float f[4] = {0.f, 0.f, 0.f, 0.f};
        if (valid)
            point_features(Gd, p, f);
        // The A operand changes layout here (K = 64 -> 16): the previous
        // tile's last rows, written by every thread in the K = 64 layout,
        // overlap other rows' K = 16 addresses, so all of them land first.
        __syncthreads();
        const uint4 h0 = make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), 0u, 0u);
        *reinterpret_cast<uint4 *>(S.a + tc::kmaj(row, 0, 2)) = h0;
        *reinterpret_cast<uint4 *>(S.a + tc::kmaj(row, 1, 2)) = make_uint4(0u, 0u, 0u, 0u);
        if (valid) {
            reinterpret_cast<uint4 *>(St.h0 + p * MLP_IN)[0] = h0;
            reinterpret_cast<uint4 *>(St.h0 + p * MLP_IN)[1] = make_uint4(0u, 0u, 0u, 0u);
        }
        // forward: Z_l in TMEM, H_l = SiLU(Z_l + b_l) stored and fed on
        const uint8_t *wf[3] = {S.w1, S.w2, S.w3};
        const float *bf[3] = {S.b1, S.b2, S.b3};
        __nv_bfloat16 *hs[3] = {St.h1, St.h2, St.h3};
#pragma unroll 1
        for (int l = 0; l < 3; ++l) {
            mma_into(64u * l, wf[l], l == 0 ? MLP_IN / 8 : MLP_H / 8, 64);
            uint32_t r[4][16];
            ld64(64u * l, r);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                float v[8];
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    v[i] = silu(__uint_as_float(r[c >> 1][(c & 1) * 8 + i]) + bf[l][8 * c + i]);
                put8(v, c, valid ? hs[l] + p * MLP_H : nullptr);
            }
        }
        // output gradient (d out_re, d out_im) as A (K = 16)
        const long long gi = valid ? gain_index(Gd, p) : -1;
        const float2 d = gi >= 0 ? dgain[gi] : make_float2(0.f, 0.f);
        const uint4 dz4 = make_uint4(pack_bf16(d.x, d.y), 0u, 0u, 0u);
        __syncthreads();  // every H3 row (K = 64 layout) is written before the K = 16 rows
        *reinterpret_cast<uint4 *>(S.a + tc::kmaj(row, 0, 2)) = dz4;
        *reinterpret_cast<uint4 *>(S.a + tc::kmaj(row, 1, 2)) = make_uint4(0u, 0u, 0u, 0u);
        if (valid) {
            reinterpret_cast<uint4 *>(St.dz4 + p * MLP_OUTP)[0] = dz4;
            reinterpret_cast<uint4 *>(St.dz4 + p * MLP_OUTP)[1] = make_uint4(0u, 0u, 0u, 0u);
        }
        // backward: dH_l = dZ_{l+1} W_{l+1} (transposed weights as B), then
        // dZ_l = dH_l * SiLU'(Z_l + b_l)
        const uint8_t *wt[3] = {S.w4t, S.w3t, S.w2t};
        __nv_bfloat16 *dzs[3] = {St.dz3, St.dz2, St.dz1};
#pragma unroll 1
        for (int k = 0; k < 3; ++k) {
            const int l = 2 - k;  // the layer whose dZ this step forms
            mma_into(192u, wt[k], k == 0 ? MLP_OUTP / 8 : MLP_H / 8, 64);
            uint32_t g[4][16], z[4][16];
            ld64(192u, g);
            ld64(64u * l, z);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                float v[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float zz = __uint_as_float(z[c >> 1][(c & 1) * 8 + i]) + bf[l][8 * c + i];
                    v[i] = __uint_as_float(g[c >> 1][(c & 1) * 8 + i]) * silu_grad_of(zz);
                }
                put8(v, c, valid ? dzs[k] + p * MLP_H : nullptr);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (*abort) {
        if (row == 0) {
            mbar_wait(&S.bar, phase ^ 1u, kTcWaitNs);
            atomicOr(&g_mlp_status, 1);
        }
        __syncthreads();
    }
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(S.tmem_base, TB_TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------
// Weight gradients of an M x N layer (M = 16*MT output rows including the
// padding, N = 8*NT inputs): dW[m][n] = sum_p DZ[p][m] H[p][n] and
// db[m] = sum_p DZ[p][m].  A CTA reduces a contiguous chunk of points; warp w
// owns output rows 16w..16w+15 and all N columns plus a column of ones (the
// bias).  Rows m >= m_valid are padding and are not written.
template <int MT, int NT>
__global__ void __launch_bounds__(32 * MT) k_mlp_wgrad(const __nv_bfloat16 *DZ, const __nv_bfloat16 *H,
                                                       long long P, long long chunk, int m_valid, float *dW,
                                                       float *db)
{
    constexpr int M = 16 * MT, N = 8 * NT;
    constexpr int LDM = M + 8, LDN = N + 8;
    __shared__ __align__(16) __nv_bfloat16 sdz[16 * LDM];
    __shared__ __align__(16) __nv_bfloat16 sh[16 * LDN];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    float acc[NT + 1][4];
#pragma unroll
    for (int nt = 0; nt <= NT; ++nt)
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
    const long long c0 = (long long)blockIdx.x * chunk;
    const long long c1 = c0 + chunk < P ? c0 + chunk : P;
    const uint32_t ones = pack_bf16(1.f, 1.f);
    const int m0 = warp * 16;
    for (long long p0 = c0; p0 < c1; p0 += 16) {
        __syncthreads();
        // 16 rows of DZ and H: contiguous, 16-byte vectors
        for (int i = threadIdx.x; i < 16 * (M / 8); i += blockDim.x) {
            const int r = i / (M / 8), c = i % (M / 8);
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (p0 + r < c1)
                v = reinterpret_cast<const uint4 *>(DZ + (p0 + r) * M)[c];
            *reinterpret_cast<uint4 *>(sdz + r * LDM + 8 * c) = v;
        }
        for (int i = threadIdx.x; i < 16 * (N / 8); i += blockDim.x) {
            const int r = i / (N / 8), c = i % (N / 8);
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (p0 + r < c1)
                v = reinterpret_cast<const uint4 *>(H + (p0 + r) * N)[c];
            *reinterpret_cast<uint4 *>(sh + r * LDN + 8 * c) = v;
        }
        __syncthreads();
        // A (M x 16 points): A[m][k] = DZ[k][m]
        uint32_t a[4];
        a[0] = pair_bf16(sdz[(2 * t) * LDM + m0 + g], sdz[(2 * t + 1) * LDM + m0 + g]);
        a[1] = pair_bf16(sdz[(2 * t) * LDM + m0 + g + 8], sdz[(2 * t + 1) * LDM + m0 + g + 8]);
        a[2] = pair_bf16(sdz[(2 * t + 8) * LDM + m0 + g], sdz[(2 * t + 9) * LDM + m0 + g]);
        a[3] = pair_bf16(sdz[(2 * t + 8) * LDM + m0 + g + 8], sdz[(2 * t + 9) * LDM + m0 + g + 8]);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            // B (16 points x N): B[k][n] = H[k][n]
            const int n = nt * 8 + g;
            const uint32_t b0 = pair_bf16(sh[(2 * t) * LDN + n], sh[(2 * t + 1) * LDN + n]);
            const uint32_t b1 = pair_bf16(sh[(2 * t + 8) * LDN + n], sh[(2 * t + 9) * LDN + n]);
            mma_bf16(acc[nt], a, b0, b1);
        }
        mma_bf16(acc[NT], a, ones, ones);
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const int n = nt * 8 + 2 * t;
        if (m0 + g < m_valid) {
            atomicAdd(dW + (size_t)(m0 + g) * N + n, acc[nt][0]);
            atomicAdd(dW + (size_t)(m0 + g) * N + n + 1, acc[nt][1]);
        }
        if (m0 + g + 8 < m_valid) {
            atomicAdd(dW + (size_t)(m0 + g + 8) * N + n, acc[nt][2]);
            atomicAdd(dW + (size_t)(m0 + g + 8) * N + n + 1, acc[nt][3]);
        }
    }
    if (t == 0) {
        if (m0 + g < m_valid)
            atomicAdd(db + m0 + g, acc[NT][0]);
        if (m0 + g + 8 < m_valid)
            atomicAdd(db + m0 + g + 8, acc[NT][2]);
    }
}

int sm_count()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
        return 1;
    return n;
}

bool aligned(const void *p, size_t a) { return ((uintptr_t)p % a) == 0; }

odt_status err(odt_status st, const std::string &msg) { return (odt_status)set_error(st, msg.c_str()); }

odt_status check_params(const odt_mlp_params *p, int32_t A, int32_t lNy, int32_t lNx, const float *feat,
                        const int32_t *positions, int32_t num_positions, MlpWeights &W, MlpGrid &Gd)
{
    if (!p || !feat)
        return err(ODT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (A < 1 || lNy < 1 || lNx < 1)
        return err(ODT_ERR_INVALID_ARGUMENT, "need num_angles, pad_ny, pad_nx >= 1");
    if (positions && (num_positions < 1 || num_positions > lNy * lNx || !aligned(positions, 4)))
        return err(ODT_ERR_INVALID_ARGUMENT, "need 1 <= num_positions <= pad_ny*pad_nx (4-byte aligned list)");
    const void *ptrs[] = {p->w1, p->w2, p->w3, p->w4, p->w2t, p->w3t, p->w4t, p->b1, p->b2, p->b3, p->b4};
    for (const void *q : ptrs)
        if (!q || !aligned(q, 16))
            return err(ODT_ERR_INVALID_ARGUMENT, "MLP weights and biases must be non-NULL and 16-byte aligned");
    if (!aligned(feat, 8))
        return err(ODT_ERR_INVALID_ARGUMENT, "angle features must be 8-byte aligned");
    W.w1 = (const __nv_bfloat16 *)p->w1;
    W.w2 = (const __nv_bfloat16 *)p->w2;
    W.w3 = (const __nv_bfloat16 *)p->w3;
    W.w4 = (const __nv_bfloat16 *)p->w4;
    W.w2t = (const __nv_bfloat16 *)p->w2t;
    W.w3t = (const __nv_bfloat16 *)p->w3t;
    W.w4t = (const __nv_bfloat16 *)p->w4t;
    W.b1 = p->b1;
    W.b2 = p->b2;
    W.b3 = p->b3;
    W.b4 = p->b4;
    Gd.A = A;
    Gd.lNy = lNy;
    Gd.lNx = lNx;
    Gd.pos = positions;
    Gd.npos = positions ? num_positions : lNy * lNx;
    Gd.P = (long long)A * Gd.npos;
    Gd.angle_feat = (const float2 *)feat;
    return ODT_OK;
}

size_t store_bytes(long long P)
{
    return (size_t)P * (MLP_IN + 3 * MLP_H + 3 * MLP_H + MLP_OUTP) * sizeof(__nv_bfloat16);
}

}  // namespace
}  // namespace odt

using namespace odt;

extern "C" {

odt_status odt_mlp_gain_forward(const odt_mlp_params *params, int32_t num_angles, int32_t pad_ny, int32_t pad_nx,
                                const float *angle_features, const int32_t *positions, int32_t num_positions,
                                void *gain, void *stream)
{
    MlpWeights W;
    MlpGrid Gd;
    odt_status st =
        check_params(params, num_angles, pad_ny, pad_nx, angle_features, positions, num_positions, W, Gd);
    if (st != ODT_OK)
        return st;
    if (!gain || !aligned(gain, 8))
        return err(ODT_ERR_INVALID_ARGUMENT, "gain must be non-NULL and 8-byte aligned");
    if (g_mlp_tensor_memory.load(std::memory_order_relaxed)) {
        static thread_local int configured_device = -1;
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess && configured_device != dev) {
            e = cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
            if (e == cudaSuccess)
                configured_device = dev;
        }
        if (e != cudaSuccess)
            return err(ODT_ERR_CUDA, std::string("k_mlp_forward_tc configuration: ") + cudaGetErrorString(e));
        // four CTAs (eight tiles in flight) per SM: shared memory and the
        // 512 TMEM columns of an SM hold four
        const long long tiles = (Gd.P + 127) / 128;
        const long long want = (tiles + TC_SLOTS - 1) / TC_SLOTS;
        const long long cap = 4LL * sm_count();
        const unsigned blocks = (unsigned)(want < cap ? want : cap);
        k_mlp_forward_tc<<<blocks, TC_THREADS, TC_SMEM, (cudaStream_t)stream>>>(W, Gd, (float2 *)gain);
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return err(ODT_ERR_CUDA, std::string("k_mlp_forward_tc: ") + cudaGetErrorString(e));
        return ODT_OK;
    }
    const long long groups = (Gd.P + 15) / 16;
    const long long want = (groups + FWD_WARPS - 1) / FWD_WARPS;
    const long long cap = 4LL * sm_count();
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    k_mlp_forward<<<blocks, 32 * FWD_WARPS, 0, (cudaStream_t)stream>>>(W, Gd, (float2 *)gain);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return err(ODT_ERR_CUDA, std::string("k_mlp_forward: ") + cudaGetErrorString(e));
    return ODT_OK;
}

odt_status odt_mlp_read_status(void *stream)
{
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    int h = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyFromSymbol(&h, g_mlp_status, sizeof(int));
    if (e == cudaSuccess && h != 0) {
        const int zero = 0;
        e = cudaMemcpyToSymbol(g_mlp_status, &zero, sizeof(int));
        if (e == cudaSuccess)
            return err(ODT_ERR_DEVICE_CHECK, "an MLP tensor-core wait gave up");
    }
    if (e != cudaSuccess)
        return err(ODT_ERR_CUDA, std::string("MLP status read: ") + cudaGetErrorString(e));
    return ODT_OK;
}

odt_status odt_mlp_store_size(int32_t num_angles, int32_t num_positions, uint64_t *bytes)
{
    if (!bytes || num_angles < 1 || num_positions < 1)
        return err(ODT_ERR_INVALID_ARGUMENT, "need num_angles, num_positions >= 1 and a result pointer");
    *bytes = store_bytes((long long)num_angles * num_positions);
    return ODT_OK;
}

odt_status odt_mlp_select_kernels(int32_t tensor_memory)
{
    if (tensor_memory != 0 && tensor_memory != 1)
        return err(ODT_ERR_INVALID_ARGUMENT, "tensor_memory must be 0 or 1");
    g_mlp_tensor_memory.store(tensor_memory, std::memory_order_relaxed);
    return ODT_OK;
}

odt_status odt_mlp_gain_backward(const odt_mlp_params *params, int32_t num_angles, int32_t pad_ny, int32_t pad_nx,
                                 const float *angle_features, const int32_t *positions, int32_t num_positions,
                                 const void *gain_grad, void *store, const odt_mlp_grads *grads, void *stream)
{
    MlpWeights W;
    MlpGrid Gd;
    odt_status st =
        check_params(params, num_angles, pad_ny, pad_nx, angle_features, positions, num_positions, W, Gd);
    if (st != ODT_OK)
        return st;
    if (!gain_grad || !aligned(gain_grad, 8) || !store || !aligned(store, 256) || !grads)
        return err(ODT_ERR_INVALID_ARGUMENT,
                   "gain_grad (8-byte aligned), store (256-byte aligned) and grads are required");
    float *outs[] = {grads->w1, grads->w2, grads->w3, grads->w4, grads->b1, grads->b2, grads->b3, grads->b4};
    for (float *q : outs)
        if (!q || !aligned(q, 4))
            return err(ODT_ERR_INVALID_ARGUMENT, "gradient buffers must be non-NULL and 4-byte aligned");
    const long long P = Gd.P;
    __nv_bfloat16 *base = reinterpret_cast<__nv_bfloat16 *>(store);
    MlpStore S;
    S.h0 = base;
    S.h1 = S.h0 + P * MLP_IN;
    S.h2 = S.h1 + P * MLP_H;
    S.h3 = S.h2 + P * MLP_H;
    S.dz1 = S.h3 + P * MLP_H;
    S.dz2 = S.dz1 + P * MLP_H;
    S.dz3 = S.dz2 + P * MLP_H;
    S.dz4 = S.dz3 + P * MLP_H;
    cudaStream_t s = (cudaStream_t)stream;
    const int sms = sm_count();
    const long long groups = (P + 15) / 16;
    const long long want = (groups + BWD_WARPS - 1) / BWD_WARPS;
    const long long cap = 4LL * sms;
    cudaError_t e = cudaSuccess;
    if (g_mlp_tensor_memory.load(std::memory_order_relaxed)) {
        static thread_local int configured_device = -1;
        int dev = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess && configured_device != dev) {
            e = cudaFuncSetAttribute(k_mlp_backward_data_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)TB_SMEM);
            if (e == cudaSuccess)
                configured_device = dev;
        }
        if (e != cudaSuccess)
            return err(ODT_ERR_CUDA, std::string("k_mlp_backward_data_tc configuration: ") + cudaGetErrorString(e));
        // two CTAs (256 TMEM columns each) per SM
        const long long tiles = (P + 127) / 128;
        const long long tcap = 2LL * sms;
        k_mlp_backward_data_tc<<<(unsigned)(tiles < tcap ? tiles : tcap), 128, TB_SMEM, s>>>(
            W, Gd, (const float2 *)gain_grad, S);
    } else {
        k_mlp_backward_data<<<(unsigned)(want < cap ? want : cap), 32 * BWD_WARPS, 0, s>>>(
            W, Gd, (const float2 *)gain_grad, S);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return err(ODT_ERR_CUDA, std::string("k_mlp_backward_data: ") + cudaGetErrorString(e));
    // split-K over the points: about two chunks per SM
    long long chunk = (P + 2LL * sms - 1) / (2LL * sms);
    chunk = (chunk + 15) / 16 * 16;
    const unsigned nchunks = (unsigned)((P + chunk - 1) / chunk);
    k_mlp_wgrad<1, 8><<<nchunks, 32, 0, s>>>(S.dz4, S.h3, P, chunk, 2, grads->w4, grads->b4);
    k_mlp_wgrad<4, 8><<<nchunks, 128, 0, s>>>(S.dz3, S.h2, P, chunk, MLP_H, grads->w3, grads->b3);
    k_mlp_wgrad<4, 8><<<nchunks, 128, 0, s>>>(S.dz2, S.h1, P, chunk, MLP_H, grads->w2, grads->b2);
    k_mlp_wgrad<4, 2><<<nchunks, 128, 0, s>>>(S.dz1, S.h0, P, chunk, MLP_H, grads->w1, grads->b1);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return err(ODT_ERR_CUDA, std::string("k_mlp_wgrad: ") + cudaGetErrorString(e));
    return ODT_OK;
}

}  // extern "C"
