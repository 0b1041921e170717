// Adjoint (vector-Jacobian product) of the filter stages, y-axis path.
//
// Forward, per angle a (stages.cu):
//   X  = FFT2(pad(w_a s_a))                          (rows, then columns)
//   V_p = G g X P_p,   P_p = exp(i w z_p) + zl_p alpha + zh_p beta
//   T_p = crop_y IFFT_y(V_p);  slab_p = L_x(T_p) = (crop_x + xfix) IFFT_x(T_p)
// with G the filter (prefilter particular factors folded in), g an optional
// real per-frequency gain, zl_p = pole^p, zh_p = pole^(nz-1-p).
//
// Adjoint, given slab_grad (from the transposed resampling, rotate.cu):
//   T_p_grad = FFT_x((crop_x + xfix)^T slab_grad_p)          k_adj_rows
//   Z_p      = FFT_y(crop_y^T T_p_grad)
//   Q        = sum_p conj(P_p) Z_p                            k_adj_columns
//   dg      += Re(conj(G X) Q)   (X recomputed)               k_adj_spectrum
//   X_grad   = conj(G g) Q;  W = IFFT_y(X_grad)               k_adj_spectrum
//   P_grad   = IFFT_x(W)                                      k_adj_rows_full
//   s_grad   = w_a pad^T(P_grad)                              k_adj_pad
// The adjoint of an unnormalised backward FFT is the unnormalised forward
// FFT and vice versa; the transpose of the x-prefilter boundary terms
// collects two weighted sums of the cotangent and scatters them onto the
// four samples outside the crop.
#include "odt_fft.cuh"
#include "odt_internal.cuh"
#include "odt_stage_util.cuh"

namespace odt {

// (a^T... ) rows: crop_x/xfix transpose + forward FFT along x.
template <class L, int LPC>
__global__ void __launch_bounds__(LPC * L::TPL) k_adj_rows(StageParams P, L line, const float2 *sgrad, float2 *Tg,
                                                           int q0, int qn)
{
    extern __shared__ float2 smem[];
    const int n = line.size();  // lNx
    const int xs = xslots<false>(n);
    float2 *buf0 = smem, *buf1 = smem + LPC * xs, *tw = smem + 2 * LPC * xs;
    float2 *red = tw + tw_slots(n);  // [LPC][2] boundary sums
    copy_twiddles<L>(tw, P.tab.twx, n);
    const int l = threadIdx.x / L::TPL, j = threadIdx.x % L::TPL;
    const int ny = P.ny, nx = P.nx, nz = P.nz, padxl = P.padxl;
    const long long rid = (long long)blockIdx.x * LPC + l;
    const bool valid = rid < (long long)qn * ny;
    const int qq = q0 + (int)((valid ? rid : 0) / ny);
    const int y = (int)((valid ? rid : 0) % ny);
    const int a = qq / nz, p = qq % nz;
    // slab gradient of (a, y, p, xx): [a][y][z][x] from the y-axis
    // resampling transpose, the forward slab layout [a][z][x][ypitch] from
    // the tilted one
    const bool tl = P.tilted != 0;
    const float2 *src = tl ? sgrad + ((size_t)a * nz + p) * nx * P.ypitch + y
                           : sgrad + (((size_t)a * ny + y) * nz + p) * nx;
    const size_t xstep = tl ? (size_t)P.ypitch : 1;
    if (threadIdx.x < 2 * LPC)
        red[threadIdx.x] = make_float2(0.f, 0.f);
    __syncthreads();
    float2 v[L::SLOTS];
    float2 gA = make_float2(0.f, 0.f), gB = make_float2(0.f, 0.f);
    const bool pf = P.order >= 2;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int x = j + r * L::TPL;
        const int xx = x - padxl;
        float2 t = make_float2(0.f, 0.f);
        if (valid && x < n && xx >= 0 && xx < nx) {
            t = src[xx * xstep];
            if (pf && xx < ZPOW_N) {
                const float zz = P.tab.zpow[xx];
                gA.x = fmaf(zz, t.x, gA.x);
                gA.y = fmaf(zz, t.y, gA.y);
            }
            if (pf && nx - 1 - xx < ZPOW_N) {
                const float zz = P.tab.zpow[nx - 1 - xx];
                gB.x = fmaf(zz, t.x, gB.x);
                gB.y = fmaf(zz, t.y, gB.y);
            }
        }
        v[r] = t;
    }
    if (pf) {
        if (gA.x != 0.f || gA.y != 0.f) {
            atomicAdd(&red[l * 2].x, gA.x);
            atomicAdd(&red[l * 2].y, gA.y);
        }
        if (gB.x != 0.f || gB.y != 0.f) {
            atomicAdd(&red[l * 2 + 1].x, gB.x);
            atomicAdd(&red[l * 2 + 1].y, gB.y);
        }
        __syncthreads();
        const float2 A = red[l * 2], B = red[l * 2 + 1];
        // d0 = u[e0] - u[e1] and d1 = u[e3] - u[e2] enter as
        // A_coef = ca d0 + cb d1, B_coef = ca d1 + cb d0
        const float2 d0g = make_float2(P.bx_ca * A.x + P.bx_cb * B.x, P.bx_ca * A.y + P.bx_cb * B.y);
        const float2 d1g = make_float2(P.bx_cb * A.x + P.bx_ca * B.x, P.bx_cb * A.y + P.bx_ca * B.y);
        const int e0 = (padxl - 1 + n) % n, e1 = (padxl + 1) % n;
        const int e2 = (padxl + nx - 2 + n) % n, e3 = (padxl + nx) % n;
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int x = j + r * L::TPL;
            if (x == e0) v[r] = v[r] + d0g;
            if (x == e1) v[r] = v[r] - d0g;
            if (x == e3) v[r] = v[r] + d1g;
            if (x == e2) v[r] = v[r] - d1g;
        }
    }
    int flip = 0;
    line.template run<-1>(v, j, buf0 + l * xs, buf1 + l * xs, 1, tw, flip);
    if (!valid)
        return;
    float2 *dst = Tg + (size_t)rid * n;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int x = j + r * L::TPL;
        if (x < n && column_active(P, x))
            dst[x] = v[r];
    }
}

// Columns: forward FFT along y of the zero-padded cotangent column of every
// plane, accumulated against the conjugate propagator into Qg[a][ky][kx].
template <class L, int KX>
__global__ void __launch_bounds__(KX * L::TPL) k_adj_columns(StageParams P, L line, const float2 *Tg, float2 *Qg,
                                                             int q0, int qn, int ppc)
{
    if (!group_active<KX>(P, blockIdx.x * KX))
        return;
    extern __shared__ float2 smem[];
    const int n = line.size();  // lNy
    const int xs = xslots<true>(n);
    float2 *buf0 = smem, *buf1 = smem + KX * xs, *tw = smem + 2 * KX * xs;
    float2 *stp = tw + tw_slots(n);  // [n][KX]
    float2 *red = stp + n * KX;      // [KX][2] y-prefilter boundary sums
    copy_twiddles<L>(tw, P.tab.twy, n);
    const int c = threadIdx.x % KX, j = threadIdx.x / KX;
    const int kx = blockIdx.x * KX + c;
    const bool colok = kx < P.lNx;
    // k_adj_rows writes the cotangent rows Tg only in the active columns;
    // a zero-band column of an active group is read as zero, never from
    // the unwritten workspace
    const bool colact = colok && column_active(P, kx);
    const int lNx = P.lNx, nz = P.nz, ny = P.ny, padyl = P.padyl;
    // tilted path: the forward's y-prefilter boundary terms (from the four
    // samples around the crop's ends) are transposed before the FFT
    const bool yfix = P.order >= 2 && P.tilted;
    const int qb = q0 + blockIdx.y * ppc;
    const int qe = min(q0 + qn, qb + ppc);
    const bool pf = P.order >= 2;
    __syncthreads();
    float2 E[L::SLOTS], Q[L::SLOTS];
    int flip = 0;
    int cur_a = -1;
    auto flush = [&](int a) {
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int ky = j + r * L::TPL;
            if (colok && ky < n) {
                float2 *d = Qg + ((size_t)a * n + ky) * lNx + kx;
                atomicAdd(&d->x, Q[r].x);
                atomicAdd(&d->y, Q[r].y);
            }
        }
    };
    int a = qb / nz, p = qb % nz;
    for (int q = qb; q < qe; ++q, ++p) {
        if (p == nz) {
            p = 0;
            ++a;
        }
        if (a != cur_a) {
            if (cur_a >= 0)
                flush(cur_a);
            const float zp = (float)p - 0.5f * (float)nz + P.zshift;
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int ky = j + r * L::TPL;
                Q[r] = make_float2(0.f, 0.f);
                if (colok && ky < n) {
                    const size_t k = (size_t)ky * lNx + kx;
                    E[r] = expi_phase(P.tab.wsplit[k], zp);
                    stp[ky * KX + c] = P.tab.step[k];
                } else {
                    E[r] = make_float2(0.f, 0.f);
                }
            }
            cur_a = a;
        }
        float2 v[L::SLOTS];
        const float2 *src = Tg + (size_t)(q - q0) * ny * lNx + kx;
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int yy = j + r * L::TPL - padyl;
            v[r] = (colact && yy >= 0 && yy < ny) ? src[(size_t)yy * lNx] : make_float2(0.f, 0.f);
        }
        if (yfix) {
            // out[yy] = u[padyl + yy] + A z^yy + B z^(ny-1-yy), with A, B from
            // d0 = u[e0] - u[e1], d1 = u[e3] - u[e2]: collect the cotangent's
            // weighted sums gA, gB over the column, then scatter
            // (ca gA + cb gB) and (cb gA + ca gB) onto the four samples
            float2 gA = make_float2(0.f, 0.f), gB = make_float2(0.f, 0.f);
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int yy = j + r * L::TPL - padyl;
                if (yy >= 0 && yy < ny) {
                    if (yy < ZPOW_N) {
                        const float zz = P.tab.zpow[yy];
                        gA = make_float2(fmaf(zz, v[r].x, gA.x), fmaf(zz, v[r].y, gA.y));
                    }
                    if (ny - 1 - yy < ZPOW_N) {
                        const float zz = P.tab.zpow[ny - 1 - yy];
                        gB = make_float2(fmaf(zz, v[r].x, gB.x), fmaf(zz, v[r].y, gB.y));
                    }
                }
            }
            __syncthreads();  // the previous plane's reads of red are done
            if (j == 0) {
                red[c * 2] = make_float2(0.f, 0.f);
                red[c * 2 + 1] = make_float2(0.f, 0.f);
            }
            __syncthreads();
            if (gA.x != 0.f || gA.y != 0.f) {
                atomicAdd(&red[c * 2].x, gA.x);
                atomicAdd(&red[c * 2].y, gA.y);
            }
            if (gB.x != 0.f || gB.y != 0.f) {
                atomicAdd(&red[c * 2 + 1].x, gB.x);
                atomicAdd(&red[c * 2 + 1].y, gB.y);
            }
            __syncthreads();
            const float2 A = red[c * 2], B = red[c * 2 + 1];
            const float2 d0g = make_float2(P.by_ca * A.x + P.by_cb * B.x, P.by_ca * A.y + P.by_cb * B.y);
            const float2 d1g = make_float2(P.by_cb * A.x + P.by_ca * B.x, P.by_cb * A.y + P.by_ca * B.y);
            const int e0 = (padyl - 1 + n) % n, e1 = (padyl + 1) % n;
            const int e2 = (padyl + ny - 2 + n) % n, e3 = (padyl + ny) % n;
#pragma unroll
            for (int r = 0; r < L::SLOTS; ++r) {
                const int yq = j + r * L::TPL;
                if (yq == e0) v[r] = v[r] + d0g;
                if (yq == e1) v[r] = v[r] - d0g;
                if (yq == e3) v[r] = v[r] + d1g;
                if (yq == e2) v[r] = v[r] - d1g;
            }
        }
        line.template run<-1, true>(v, j, buf0 + c, buf1 + c, KX, tw, flip);
        const float zl = (pf && p < ZPOW_N) ? P.tab.zpow[p] : 0.f;
        const float zh = (pf && nz - 1 - p < ZPOW_N) ? P.tab.zpow[nz - 1 - p] : 0.f;
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int ky = j + r * L::TPL;
            // conj(P_p) Z = conj(E) Z + zl conj(alpha) Z + zh conj(beta) Z
            const float2 e = E[r];
            float2 cz = make_float2(fmaf(e.x, v[r].x, e.y * v[r].y), fmaf(e.x, v[r].y, -e.y * v[r].x));
            if ((zl != 0.f || zh != 0.f) && colok && ky < n) {
                const size_t k = (size_t)ky * lNx + kx;
                float2 b = make_float2(0.f, 0.f);
                if (zl != 0.f) {
                    const float2 al = P.tab.alpha[k];
                    b = make_float2(zl * al.x, zl * al.y);
                }
                if (zh != 0.f) {
                    const float2 be = P.tab.beta[k];
                    b = make_float2(fmaf(zh, be.x, b.x), fmaf(zh, be.y, b.y));
                }
                cz.x = fmaf(b.x, v[r].x, fmaf(b.y, v[r].y, cz.x));
                cz.y = fmaf(b.x, v[r].y, fmaf(-b.y, v[r].x, cz.y));
            }
            Q[r] = Q[r] + cz;
            if (ky < n)
                E[r] = cmul(E[r], stp[ky * KX + c]);
        }
    }
    if (cur_a >= 0)
        flush(cur_a);
}

// Spectrum: gain gradient dg += Re(conj(G X) Q) (X recomputed from the row
// spectra), then W = IFFT_y(conj(G g) Q) for every padded row.
template <class L, int KX>
__global__ void __launch_bounds__(KX * L::TPL) k_adj_spectrum(StageParams P, L line, const float2 *rowspec,
                                                              const float2 *Qg, float *dgain, float2 *dagain,
                                                              float2 *W)
{
    if (!group_active<KX>(P, blockIdx.x * KX))
        return;
    extern __shared__ float2 smem[];
    const int n = line.size();  // lNy
    const int xs = xslots<true>(n);
    float2 *buf0 = smem, *buf1 = smem + KX * xs, *tw = smem + 2 * KX * xs;
    copy_twiddles<L>(tw, P.tab.twy, n);
    const int c = threadIdx.x % KX, j = threadIdx.x / KX;
    const int kx = blockIdx.x * KX + c;
    const bool colok = kx < P.lNx;
    const int lNx = P.lNx;
    const int a = blockIdx.y;
    __syncthreads();
    int flip = 0;
    float2 X[L::SLOTS];
    const bool need_x = dgain || dagain;
    if (need_x) {
#pragma unroll
        for (int r = 0; r < L::SLOTS; ++r) {
            const int ky = j + r * L::TPL;
            X[r] = (colok && ky < n) ? rowspec[((size_t)a * n + ky) * lNx + kx] : make_float2(0.f, 0.f);
        }
        line.template run<-1, true>(X, j, buf0 + c, buf1 + c, KX, tw, flip);
    }
    float2 v[L::SLOTS];
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int ky = j + r * L::TPL;
        v[r] = make_float2(0.f, 0.f);
        if (colok && ky < n) {
            const size_t k = (size_t)ky * lNx + kx;
            const float2 q = Qg[((size_t)a * n + ky) * lNx + kx];
            const float2 G = P.tab.G[k];
            const float gk = P.gain ? P.gain[k] : 1.f;
            const size_t ak = (size_t)a * n * lNx + k;
            const float2 ga = P.again ? P.again[ak] : make_float2(1.f, 0.f);
            if (dgain) {
                // d/dg of G g ga X: Re(conj(G ga X) q)
                const float2 gx = cmul(cmul(G, ga), X[r]);
                atomicAdd(dgain + k, gx.x * q.x + gx.y * q.y);
            }
            if (dagain) {
                // d/d(ga) of G g ga X: conj(G g X) q
                const float2 gx = cscale(cmul(G, X[r]), gk);
                dagain[ak] = make_float2(gx.x * q.x + gx.y * q.y, gx.x * q.y - gx.y * q.x);
            }
            // conj(G g ga) q
            const float2 h = cscale(cmul(G, ga), gk);
            v[r] = make_float2(h.x * q.x + h.y * q.y, h.x * q.y - h.y * q.x);
        }
    }
    line.template run<1, true>(v, j, buf0 + c, buf1 + c, KX, tw, flip);
    if (!colok)
        return;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int ky = j + r * L::TPL;
        if (ky < n)
            W[((size_t)a * n + ky) * lNx + kx] = v[r];
    }
}

// Rows: full backward FFT along x of W -> the cotangent of the padded plane.
template <class L, int LPC>
__global__ void __launch_bounds__(LPC * L::TPL) k_adj_rows_full(StageParams P, L line, const float2 *W, float2 *Pg,
                                                                int nb)
{
    extern __shared__ float2 smem[];
    const int n = line.size();  // lNx
    const int xs = xslots<false>(n);
    float2 *buf0 = smem, *buf1 = smem + LPC * xs, *tw = smem + 2 * LPC * xs;
    copy_twiddles<L>(tw, P.tab.twx, n);
    const int l = threadIdx.x / L::TPL, j = threadIdx.x % L::TPL;
    const long long lid = (long long)blockIdx.x * LPC + l;
    const bool valid = lid < (long long)nb * P.lNy;
    const float2 *src = W + (size_t)(valid ? lid : 0) * n;
    float2 v[L::SLOTS];
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int x = j + r * L::TPL;
        v[r] = (valid && x < n && column_active(P, x)) ? src[x] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    int flip = 0;
    line.template run<1>(v, j, buf0 + l * xs, buf1 + l * xs, 1, tw, flip);
    if (!valid)
        return;
    float2 *dst = Pg + (size_t)lid * n;
#pragma unroll
    for (int r = 0; r < L::SLOTS; ++r) {
        const int x = j + r * L::TPL;
        if (x < n)
            dst[x] = v[r];
    }
}

// Transpose of the padding along one axis: the padded positions that a
// source index contributes to, with their coefficients (1 for data and
// edge padding, the ramp fraction for linear_ramp).
struct PadAxis {
    int n, pad_l, pad_r, mode;  // mode: 0 none, 1 edge, 2 ramp
};

template <class F>
__device__ __forceinline__ void pad_transpose_axis(const PadAxis &ax, int i, F &&emit)
{
    emit(i + ax.pad_l, 1.f);
    if (ax.mode == 0)
        return;
    if (i == 0) {
        for (int q = 0; q < ax.pad_l; ++q)
            emit(q, ax.mode == 1 ? 1.f : (float)q / (float)ax.pad_l);
    }
    if (i == ax.n - 1) {
        for (int jj = 0; jj < ax.pad_r; ++jj)
            emit(ax.pad_l + ax.n + jj, ax.mode == 1 ? 1.f : (float)(ax.pad_r - 1 - jj) / (float)ax.pad_r);
    }
}

__global__ void k_adj_pad(StageParams P, const float2 *Pg, const double *weights, int nb, float2 *dsino)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int a = blockIdx.z;
    if (x >= P.nx || a >= nb)
        return;
    const PadAxis ay{P.ny, P.padyl, P.lNy - P.ny - P.padyl, P.pad_mode};
    const PadAxis axx{P.nx, P.padxl, P.lNx - P.nx - P.padxl, P.pad_mode};
    const float2 *plane = Pg + (size_t)a * P.lNy * P.lNx;
    float2 acc = make_float2(0.f, 0.f);
    pad_transpose_axis(ay, y, [&](int Y, float cy) {
        pad_transpose_axis(axx, x, [&](int X, float cx) {
            const float2 g = plane[(size_t)Y * P.lNx + X];
            const float cc = cy * cx;
            acc.x = fmaf(cc, g.x, acc.x);
            acc.y = fmaf(cc, g.y, acc.y);
        });
    });
    const float w = weights ? (float)weights[a] : 1.f;
    dsino[((size_t)a * P.ny + y) * P.nx + x] = make_float2(w * acc.x, w * acc.y);
}

// ---------------------------------------------------------------------------
constexpr int kAdjPlanesPerBlock = 16;

template <class L>
static size_t smem_adj_rows(int n)
{
    return (size_t)(2 * Cfg<L>::LPC * xslots<false>(n) + tw_slots(n) + 2 * Cfg<L>::LPC) * sizeof(float2);
}
template <class L>
static size_t smem_adj_cols(int n)
{
    return (size_t)(2 * Cfg<L>::KX * xslots<true>(n) + Cfg<L>::KX * n + tw_slots(n) + 2 * Cfg<L>::KX) *
           sizeof(float2);
}

template <class L>
static cudaError_t set_adj_attrs(int n)
{
    if (std::is_same<L, GenericLine>::value)
        n = GenericLine::TPL * GenericLine::SLOTS;
    cudaError_t e;
    e = cudaFuncSetAttribute(k_adj_rows<L, Cfg<L>::LPC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_adj_rows<L>(n));
    if (e != cudaSuccess)
        return e;
    e = cudaFuncSetAttribute(k_adj_rows_full<L, Cfg<L>::LPC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_adj_rows<L>(n));
    if (e != cudaSuccess)
        return e;
    e = cudaFuncSetAttribute(k_adj_columns<L, Cfg<L>::KX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_adj_cols<L>(n));
    if (e != cudaSuccess)
        return e;
    return cudaFuncSetAttribute(k_adj_spectrum<L, Cfg<L>::KX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem_adj_cols<L>(n));
}

cudaError_t configure_adjoint_kernels(const StageParams &P)
{
    cudaError_t e = with_line(P.lNx, [&](auto line) { return set_adj_attrs<decltype(line)>(line.n); });
    if (e != cudaSuccess)
        return e;
    return with_line(P.lNy, [&](auto line) { return set_adj_attrs<decltype(line)>(line.n); });
}

cudaError_t launch_adj_rows(const StageParams &P, const float2 *sgrad, float2 *Tg, int q0, int qn, cudaStream_t s)
{
    return with_line(P.lNx, [&](auto line) {
        using L = decltype(line);
        constexpr int LPC = Cfg<L>::LPC;
        const long long lines = (long long)qn * P.ny;
        k_adj_rows<L, LPC><<<(unsigned)((lines + LPC - 1) / LPC), LPC * L::TPL, smem_adj_rows<L>(line.n), s>>>(
            P, line, sgrad, Tg, q0, qn);
        return cudaGetLastError();
    });
}

cudaError_t launch_adj_columns(const StageParams &P, const float2 *Tg, float2 *Qg, int q0, int qn, cudaStream_t s)
{
    return with_line(P.lNy, [&](auto line) {
        using L = decltype(line);
        constexpr int KX = Cfg<L>::KX;
        dim3 grid((P.lNx + KX - 1) / KX, (qn + kAdjPlanesPerBlock - 1) / kAdjPlanesPerBlock);
        k_adj_columns<L, KX><<<grid, KX * L::TPL, smem_adj_cols<L>(line.n), s>>>(P, line, Tg, Qg, q0, qn,
                                                                                kAdjPlanesPerBlock);
        return cudaGetLastError();
    });
}

cudaError_t launch_adj_spectrum(const StageParams &P, const float2 *rowspec, const float2 *Qg, float *dgain,
                                float2 *dagain, float2 *W, int nb, cudaStream_t s)
{
    return with_line(P.lNy, [&](auto line) {
        using L = decltype(line);
        constexpr int KX = Cfg<L>::KX;
        dim3 grid((P.lNx + KX - 1) / KX, nb);
        k_adj_spectrum<L, KX><<<grid, KX * L::TPL, smem_adj_cols<L>(line.n), s>>>(P, line, rowspec, Qg, dgain,
                                                                                 dagain, W);
        return cudaGetLastError();
    });
}

cudaError_t launch_adj_rows_full(const StageParams &P, const float2 *W, float2 *Pg, int nb, cudaStream_t s)
{
    return with_line(P.lNx, [&](auto line) {
        using L = decltype(line);
        constexpr int LPC = Cfg<L>::LPC;
        const long long lines = (long long)nb * P.lNy;
        k_adj_rows_full<L, LPC><<<(unsigned)((lines + LPC - 1) / LPC), LPC * L::TPL, smem_adj_rows<L>(line.n),
                                  s>>>(P, line, W, Pg, nb);
        return cudaGetLastError();
    });
}

cudaError_t launch_adj_pad(const StageParams &P, const float2 *Pg, const double *weights, int nb, float2 *dsino,
                           cudaStream_t s)
{
    dim3 grid((P.nx + 127) / 128, P.ny, nb);
    k_adj_pad<<<grid, 128, 0, s>>>(P, Pg, weights, nb, dsino);
    return cudaGetLastError();
}

}  // namespace odt
