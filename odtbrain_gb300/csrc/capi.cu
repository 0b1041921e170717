// C ABI of odtbrain_gb300 (declared in include/odtbrain_gb300.h).
//
// Plan creation turns the FP64 host constants of the reference
// (odtbrain/_alg3d_bpp.py:317-437; _alg3d_bppt.py:680-820) into the FP32
// device tables the stage kernels read, and sizes the angle batches.
// Execution runs, per batch of angles, the filter stages into coefficient
// slabs and then the resampling/accumulation stage.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/odtbrain_gb300.h"
#include "odt_internal.cuh"

using odt::FilterTables;
using odt::RotParams;
using odt::StageParams;

namespace {

thread_local std::string g_last_error;

odt_status fail(odt_status st, const std::string &msg)
{
    g_last_error = msg;
    return st;
}

odt_status cuda_fail(cudaError_t e, const char *where)
{
    return fail(ODT_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Test hook (odt_debug_set_table_alloc_limit): plan creation refuses table
// allocations above this many bytes (0: no limit).
uint64_t g_table_alloc_limit = 0;
std::mutex g_debug_mutex;

constexpr uint64_t kDefaultWorkspace = 16ull << 30;   // 16 GiB of slabs, chunk buffers etc.
// column-stage output chunks: two buffers of half this size in total.  Large
// chunks (1024 planes of a 512-wide spectrum per buffer) mean few launches
// with full waves; measured on the 256^3 workload: 64 MB 92.8 ms, 256 MB
// 84.2 ms, 1 GB 79.3 ms, 2 GB 78.7 ms, 4 GB 78.7 ms per reconstruction.
constexpr uint64_t kPlaneBudget = 2048ull << 20;
constexpr size_t kAlign = 256;

size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// The sampled centred B-spline of order 2..5, t[0] + t[1] (z + 1/z) +
// t[2] (z^2 + 1/z^2): [1 6 1]/8, [1 4 1]/6, [1 76 230 76 1]/384,
// [1 26 66 26 1]/120 (the kernel scipy.ndimage's prefilter inverts).
struct SplineTaps {
    double t[3];
    int npoles;  // 1 for orders 2, 3; 2 for orders 4, 5
};
SplineTaps spline_taps(int order)
{
    switch (order) {
    case 2: return {{6.0 / 8.0, 1.0 / 8.0, 0.0}, 1};
    case 3: return {{4.0 / 6.0, 1.0 / 6.0, 0.0}, 1};
    case 4: return {{230.0 / 384.0, 76.0 / 384.0, 1.0 / 384.0}, 2};
    default: return {{66.0 / 120.0, 26.0 / 120.0, 1.0 / 120.0}, 2};
    }
}

// Transfer function Bhat(w) of the sampled B-spline.
double spline_bhat(int order, double w)
{
    const SplineTaps T = spline_taps(order);
    return T.t[0] + 2.0 * T.t[1] * std::cos(w) + 2.0 * T.t[2] * std::cos(2.0 * w);
}

// Poles of the prefilter (the roots of the kernel's polynomial inside the
// unit circle), largest magnitude first.
int spline_poles(int order, double *z)
{
    const SplineTaps T = spline_taps(order);
    if (T.npoles == 1) {
        // t1 z^2 + t0 z + t1 = 0
        z[0] = (-T.t[0] + std::sqrt(T.t[0] * T.t[0] - 4.0 * T.t[1] * T.t[1])) / (2.0 * T.t[1]);
        return 1;
    }
    // with s = z + 1/z: t2 s^2 + t1 s + (t0 - 2 t2) = 0, then z^2 - s z + 1 = 0;
    // the root inside the unit circle as 2 / (s - sqrt(s^2 - 4)) (s < -2)
    const double disc = std::sqrt(T.t[1] * T.t[1] - 4.0 * T.t[2] * (T.t[0] - 2.0 * T.t[2]));
    const double s1 = (-T.t[1] + disc) / (2.0 * T.t[2]), s2 = (-T.t[1] - disc) / (2.0 * T.t[2]);
    z[0] = 2.0 / (s1 - std::sqrt(s1 * s1 - 4.0));
    z[1] = 2.0 / (s2 - std::sqrt(s2 * s2 - 4.0));
    return 2;
}

// Boundary solve of the prefilter folded into the transforms.  A line of n
// samples whose Fourier components were divided by Bhat (the particular
// solution c_p, known also beyond the line's ends) becomes scipy's
// mirror-boundary prefiltered line c = c_p + h with
//   h[k] = sum_i A_i z_i^k + B_i z_i^(n-1-k),
// where the coefficients follow from the kernel's equations at the first
// and last npoles samples, written with mirrored neighbours:
//   (A_1..A_np, B_1..B_np) = K (d_1L..d_npL, d_1R..d_npR),
//   d_mL = c_p[m] - c_p[-m],   d_mR = c_p[n-1-m] - c_p[n-1+m].
// K (row-major, 2np x 2np) is returned; false if the system is singular.
bool boundary_matrix(int order, int n, double *K)
{
    const SplineTaps T = spline_taps(order);
    double z[2];
    const int np = spline_poles(order, z), n2 = 2 * np;
    double M[4][4] = {}, R[4][4] = {};
    auto mirror = [&](int m) {
        if (n == 1)
            return 0;
        const int P = 2 * n - 2;
        m = std::abs(m) % P;
        return m < n ? m : P - m;
    };
    auto add_h = [&](int eq, double t, int k) {  // t * h[k]
        for (int i = 0; i < np; ++i) {
            M[eq][i] += t * std::pow(z[i], k);
            M[eq][np + i] += t * std::pow(z[i], n - 1 - k);
        }
    };
    int eq = 0;
    for (int q = 0; q < np; ++q, ++eq) {  // samples q (left) ...
        for (int k = -np; k <= np; ++k) {
            const int m = q + k;
            add_h(eq, T.t[std::abs(k)], mirror(m));
            if (m < 0)
                R[eq][-m - 1] -= T.t[std::abs(k)];
        }
    }
    for (int q = 0; q < np; ++q, ++eq) {  // ... and n-1-q (right)
        for (int k = -np; k <= np; ++k) {
            const int m = n - 1 - q + k;
            add_h(eq, T.t[std::abs(k)], mirror(m));
            if (m > n - 1)
                R[eq][np + (m - (n - 1)) - 1] -= T.t[std::abs(k)];
        }
    }
    // K = M^-1 R by Gauss-Jordan elimination with partial pivoting
    for (int c = 0; c < n2; ++c) {
        int piv = c;
        for (int r = c + 1; r < n2; ++r)
            if (std::fabs(M[r][c]) > std::fabs(M[piv][c]))
                piv = r;
        if (!(std::fabs(M[piv][c]) > 1e-300))
            return false;
        for (int j = 0; j < n2; ++j) {
            std::swap(M[c][j], M[piv][j]);
            std::swap(R[c][j], R[piv][j]);
        }
        const double inv = 1.0 / M[c][c];
        for (int j = 0; j < n2; ++j) {
            M[c][j] *= inv;
            R[c][j] *= inv;
        }
        for (int r = 0; r < n2; ++r) {
            if (r == c)
                continue;
            const double f = M[r][c];
            for (int j = 0; j < n2; ++j) {
                M[r][j] -= f * M[c][j];
                R[r][j] -= f * R[c][j];
            }
        }
    }
    for (int r = 0; r < n2; ++r)
        for (int j = 0; j < n2; ++j) {
            K[r * n2 + j] = R[r][j];
            if (!std::isfinite(R[r][j]))
                return false;
        }
    return true;
}

// Coefficients of the one-pole boundary solve in the form the adjoint
// kernels use: with d0 = u[-1] - u[1] and d1 = u[n] - u[n-2], the
// correction A z^k + B z^(n-1-k) has A = ca*d0 + cb*d1 and B = ca*d1 + cb*d0.
void boundary_solve(double z, int n, double *ca, double *cb)
{
    const double a = z - 1.0 / z;
    const double b = std::pow(z, n - 2) - std::pow(z, n);
    const double det = a * a - b * b;
    *ca = a / det;
    *cb = -b / det;
}

double fftfreq_rad(int k, int n)
{
    // 2*pi*numpy.fft.fftfreq(n)[k]
    const int half = (n - 1) / 2;
    const int m = k <= half ? k : k - n;
    return 2.0 * M_PI * (double)m / (double)n;
}

}  // namespace

int odt::set_error(int status, const char *msg)
{
    return (int)fail((odt_status)status, msg ? msg : "");
}

struct odt_bpp3d_plan {
    odt_bpp3d_desc d;
    int device;      // CUDA device the tables, events and stream belong to
    int nz;
    int batch;       // angles per batch
    int jobs;        // (angle, plane) jobs per column/row launch
    int ydefer;      // the row stage adds the y-prefilter terms (StageParams::ydefer)
    size_t off_rowspec, off_T, off_T2, off_Tab, off_slab, off_comp, off_rot, ws_bytes;
    size_t off_Qg, off_W, off_Pg, off_vT, adj_ws_bytes;  // adjoint-only regions after ws_bytes
    double bx_ca, bx_cb, by_ca, by_cb;  // one-pole solve in the adjoint's form
    int npoles;                         // prefilter poles: 0, 1 or 2
    float kx_solve[16], ky_solve[16];   // boundary_matrix of x and y lines
    int kx_zero_lo, kx_zero_hi;  // all-zero spectrum columns [lo, hi)
    int col_slots;               // resident column-stage CTAs (occupancy x SMs)
    // device tables (one allocation)
    void *d_tables;
    FilterTables tab;
    int *d_status;
    // chunk pipeline: the row stage of chunk k runs on s2 while the column
    // stage of chunk k+1 runs on the caller's stream (two column-stage
    // output buffers, ordered by events)
    cudaStream_t s2;
    cudaEvent_t ev_fork, ev_join, ev_col[2], ev_row[2];
};

namespace {

// The plan's device must be the current one: its tables, events and second
// stream belong to that device.
odt_status check_device(const odt_bpp3d_plan *plan)
{
    int dev = -1;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (dev != plan->device) {
        char buf[128];
        snprintf(buf, sizeof buf, "plan was created on CUDA device %d but device %d is current", plan->device,
                 dev);
        return fail(ODT_ERR_INVALID_ARGUMENT, buf);
    }
    return ODT_OK;
}

void destroy_sync_objects(odt_bpp3d_plan *p)
{
    if (p->s2)
        cudaStreamDestroy(p->s2);
    for (cudaEvent_t ev : {p->ev_fork, p->ev_join, p->ev_col[0], p->ev_col[1], p->ev_row[0], p->ev_row[1]})
        if (ev)
            cudaEventDestroy(ev);
    p->s2 = nullptr;
}

StageParams stage_params(const odt_bpp3d_plan *p)
{
    StageParams P;
    const odt_bpp3d_desc &d = p->d;
    P.A = d.num_angles;
    P.ny = d.ny;
    P.nx = d.nx;
    P.nz = p->nz;
    P.lNy = d.pad_ny;
    P.lNx = d.pad_nx;
    P.padyl = d.pad_y_left;
    P.padxl = d.pad_x_left;
    P.pad_mode = d.pad_mode;
    P.padval = make_float2((float)d.padval_re, (float)d.padval_im);
    P.order = d.intp_order;
    P.tilted = d.geometry == ODT_GEOM_AFFINE3D;
    P.in_c128 = d.input_dtype == ODT_INPUT_C128;
    P.kx_zero_lo = p->kx_zero_lo;
    P.kx_zero_hi = p->kx_zero_hi;
    P.bx_ca = (float)p->bx_ca;
    P.bx_cb = (float)p->bx_cb;
    P.by_ca = (float)p->by_ca;
    P.by_cb = (float)p->by_cb;
    P.npoles = p->npoles;
    for (int i = 0; i < 16; ++i) {
        P.kxs[i] = p->kx_solve[i];
        P.kys[i] = p->ky_solve[i];
    }
    P.ypitch = odt::yaxis_slab_pitch(d.ny);
    P.col_slots = p->col_slots;
    P.zshift = (float)d.z_shift;
    P.tab = p->tab;
    P.gain = nullptr;
    P.again = nullptr;
    P.status = p->d_status;
    P.ydefer = p->ydefer;
    P.yedge_off = p->ydefer ? (long long)p->jobs * d.ny * d.pad_nx : 0;
    return P;
}

odt_status validate(const odt_bpp3d_desc *d)
{
    if (!d)
        return fail(ODT_ERR_INVALID_ARGUMENT, "descriptor is NULL");
    if (d->num_angles < 1 || d->ny < 1 || d->nx < 2)
        return fail(ODT_ERR_INVALID_ARGUMENT, "need num_angles >= 1, ny >= 1, nx >= 2");
    if (d->pad_ny < d->ny || d->pad_nx < d->nx || d->pad_y_left < 0 || d->pad_x_left < 0 ||
        d->pad_y_left + d->ny > d->pad_ny || d->pad_x_left + d->nx > d->pad_nx)
        return fail(ODT_ERR_INVALID_ARGUMENT, "inconsistent padding geometry");
    if (d->pad_mode < ODT_PAD_NONE || d->pad_mode > ODT_PAD_RAMP)
        return fail(ODT_ERR_INVALID_ARGUMENT, "unknown pad_mode");
    if (d->pad_mode == ODT_PAD_NONE && (d->pad_ny != d->ny || d->pad_nx != d->nx))
        return fail(ODT_ERR_INVALID_ARGUMENT, "pad_mode NONE needs unpadded sizes");
    if (d->geometry != ODT_GEOM_Y_AXIS && d->geometry != ODT_GEOM_AFFINE3D)
        return fail(ODT_ERR_INVALID_ARGUMENT, "unknown geometry");
    if (d->input_dtype != ODT_INPUT_C64 && d->input_dtype != ODT_INPUT_C128)
        return fail(ODT_ERR_INVALID_ARGUMENT, "unknown input dtype");
    if (d->intp_order < 0 || d->intp_order > 5)
        return fail(ODT_ERR_INVALID_ARGUMENT, "intp_order must be in 0..5");
    if (d->intp_order >= 4 && (d->nx < 4 || (d->geometry == ODT_GEOM_AFFINE3D && d->ny > 1 && d->ny < 4)))
        return fail(ODT_ERR_UNSUPPORTED, "spline orders 4 and 5 need lines of at least 4 samples");
    if (!std::isfinite(d->z_shift) || std::fabs(d->z_shift) > 1.0 || 2.0 * d->z_shift != std::rint(2.0 * d->z_shift))
        return fail(ODT_ERR_INVALID_ARGUMENT, "z_shift must be 0, +-0.5 or +-1");
    if (!odt::line_size_supported(d->pad_nx) || !odt::line_size_supported(d->pad_ny))
        return fail(ODT_ERR_UNSUPPORTED,
                    "FFT length must be a power of two in [64, 4096] or any length <= 1024");
    if (!d->filter || !d->kz_phase)
        return fail(ODT_ERR_INVALID_ARGUMENT, "filter and kz_phase tables are required");
    // the resampling kernels address one angle's slab [z][x][y pitch] with
    // 32-bit element offsets
    if ((long long)d->nx * d->nx * odt::yaxis_slab_pitch(d->ny) >= (1ll << 31))
        return fail(ODT_ERR_UNSUPPORTED, "one angle's coefficient slab must hold fewer than 2^31 elements");
    return ODT_OK;
}

}  // namespace

extern "C" {

const char *odt_status_string(odt_status s)
{
    switch (s) {
    case ODT_OK: return "ok";
    case ODT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case ODT_ERR_UNSUPPORTED: return "unsupported";
    case ODT_ERR_CUDA: return "CUDA error";
    case ODT_ERR_OUT_OF_MEMORY: return "out of memory";
    case ODT_ERR_DEVICE_CHECK: return "device-side check failed";
    }
    return "unknown status";
}

const char *odt_last_error(void) { return g_last_error.c_str(); }

odt_status odt_bpp3d_plan_create(const odt_bpp3d_desc *desc, odt_bpp3d_plan **out)
{
    if (!out)
        return fail(ODT_ERR_INVALID_ARGUMENT, "plan output pointer is NULL");
    *out = nullptr;
    odt_status st = validate(desc);
    if (st != ODT_OK)
        return st;
    odt_bpp3d_plan *p = new (std::nothrow) odt_bpp3d_plan();
    if (!p)
        return fail(ODT_ERR_OUT_OF_MEMORY, "host allocation failed");
    p->d = *desc;
    p->d.filter = nullptr;
    p->d.kz_phase = nullptr;
    const odt_bpp3d_desc &d = p->d;
    const int lNy = d.pad_ny, lNx = d.pad_nx, nz = d.nx;
    p->nz = nz;
    const int order = d.intp_order;
    const bool pf = order >= 2;
    const bool tilted = d.geometry == ODT_GEOM_AFFINE3D;
    const size_t K = (size_t)lNy * lNx;

    // ---- FP64 host tables -> FP32 device tables
    // prefilter (order >= 2): npoles poles; per pole the z-boundary tables
    // alpha_i, beta_i (planes) and the powers z_i^m
    double zpole[2] = {0.0, 0.0};
    const int np = pf ? spline_poles(order, zpole) : 0;
    p->npoles = np;
    std::vector<float2> G(K), W(K), S(K), AL((size_t)2 * K), BE((size_t)2 * K), twx(lNx), twy(lNy);
    std::vector<float> zp((size_t)2 * odt::ZPOW_N, 0.f);
    double Kz[16] = {0}, Kx[16] = {0}, Ky[16] = {0};
    std::memset(p->kx_solve, 0, sizeof p->kx_solve);
    std::memset(p->ky_solve, 0, sizeof p->ky_solve);
    if (pf) {
        bool ok = boundary_matrix(order, nz, Kz) && boundary_matrix(order, d.nx, Kx);
        if (d.ny >= 2)
            ok = ok && boundary_matrix(order, d.ny, Ky);
        if (!ok) {
            delete p;
            return fail(ODT_ERR_UNSUPPORTED, "the spline prefilter's boundary system is singular for these sizes");
        }
        for (int i = 0; i < 16; ++i) {
            p->kx_solve[i] = (float)Kx[i];
            p->ky_solve[i] = (float)Ky[i];
        }
        if (np == 1) {
            // the adjoint kernels' form of the one-pole solve
            boundary_solve(zpole[0], d.nx, &p->bx_ca, &p->bx_cb);
            if (d.ny >= 2)
                boundary_solve(zpole[0], d.ny, &p->by_ca, &p->by_cb);
        }
        for (int i = 0; i < np; ++i) {
            double zz = 1.0;
            for (int m = 0; m < odt::ZPOW_N; ++m) {
                zp[(size_t)i * odt::ZPOW_N + m] = (float)zz;
                zz *= zpole[i];
            }
        }
    }
    // positions of the first and last planes (the z-prefilter boundary terms
    // are per-frequency functions of them)
    const double z_first = 0.0 - 0.5 * nz + d.z_shift, z_last = (double)(nz - 1) - 0.5 * nz + d.z_shift;
    for (int ky = 0; ky < lNy; ++ky) {
        // (scipy leaves an axis of length 1 unfiltered: no y prefilter, and
        // its boundary coefficients stay zero, for a single detector row)
        const double iby = (pf && tilted && d.ny >= 2) ? 1.0 / spline_bhat(order, fftfreq_rad(ky, lNy)) : 1.0;
        for (int kx = 0; kx < lNx; ++kx) {
            const size_t k = (size_t)ky * lNx + kx;
            const double ibx = pf ? 1.0 / spline_bhat(order, fftfreq_rad(kx, lNx)) : 1.0;
            const double w = desc->kz_phase[k];
            const double ibw = pf ? 1.0 / spline_bhat(order, w) : 1.0;
            const double sc = ibx * iby * ibw;
            G[k] = make_float2((float)(desc->filter[2 * k] * sc), (float)(desc->filter[2 * k + 1] * sc));
            const float whi = (float)w;
            W[k] = make_float2(whi, (float)(w - (double)whi));
            S[k] = make_float2((float)std::cos(w), (float)std::sin(w));
            for (int i = 0; i < 2; ++i) {
                AL[(size_t)i * K + k] = make_float2(0.f, 0.f);
                BE[(size_t)i * K + k] = make_float2(0.f, 0.f);
            }
            if (pf) {
                // along z the particular solution of plane p is exp(i w z_p):
                // d_mL = e(z_first) 2i sin(m w), d_mR = -e(z_last) 2i sin(m w)
                const std::complex<double> I(0.0, 1.0);
                const std::complex<double> e0 = std::exp(I * (w * z_first));
                const std::complex<double> en = std::exp(I * (w * z_last));
                std::complex<double> dv[4];
                for (int m = 1; m <= np; ++m) {
                    dv[m - 1] = e0 * (2.0 * std::sin(m * w)) * I;
                    dv[np + m - 1] = en * (-2.0 * std::sin(m * w)) * I;
                }
                const int n2 = 2 * np;
                for (int r = 0; r < n2; ++r) {
                    std::complex<double> c = 0.0;
                    for (int j = 0; j < n2; ++j)
                        c += Kz[r * n2 + j] * dv[j];
                    const float2 cf = make_float2((float)c.real(), (float)c.imag());
                    if (r < np)
                        AL[(size_t)r * K + k] = cf;
                    else
                        BE[(size_t)(r - np) * K + k] = cf;
                }
            }
        }
    }
    // largest run of all-zero filter columns around the Nyquist column
    // (outside the |k| < km disc): neither computed nor read
    {
        auto zero_col = [&](int kx) {
            for (int ky = 0; ky < lNy; ++ky) {
                const size_t k = (size_t)ky * lNx + kx;
                if (desc->filter[2 * k] != 0.0 || desc->filter[2 * k + 1] != 0.0)
                    return false;
            }
            return true;
        };
        int lo = lNx / 2, hi = lNx / 2;
        if (zero_col(lNx / 2)) {
            hi = lNx / 2 + 1;
            while (lo > 0 && zero_col(lo - 1))
                --lo;
            while (hi < lNx && zero_col(hi))
                ++hi;
        }
        p->kx_zero_lo = lo;
        p->kx_zero_hi = hi;
    }
    for (int m = 0; m < lNx; ++m)
        twx[m] = make_float2((float)std::cos(-2.0 * M_PI * m / lNx), (float)std::sin(-2.0 * M_PI * m / lNx));
    for (int m = 0; m < lNy; ++m)
        twy[m] = make_float2((float)std::cos(-2.0 * M_PI * m / lNy), (float)std::sin(-2.0 * M_PI * m / lNy));

    size_t o = 0;
    const size_t oG = o; o = align_up(o + K * 8);
    const size_t oW = o; o = align_up(o + K * 8);
    const size_t oS = o; o = align_up(o + K * 8);
    const size_t oA = o; o = align_up(o + 2 * K * 8);
    const size_t oB = o; o = align_up(o + 2 * K * 8);
    const size_t oTx = o; o = align_up(o + (size_t)lNx * 8);
    const size_t oTy = o; o = align_up(o + (size_t)lNy * 8);
    const size_t oZ = o; o = align_up(o + 2 * odt::ZPOW_N * 4);
    const size_t oSt = o; o = align_up(o + 16);
    {
        std::lock_guard<std::mutex> lock(g_debug_mutex);
        if (g_table_alloc_limit && o > g_table_alloc_limit) {
            delete p;
            return fail(ODT_ERR_OUT_OF_MEMORY, "plan tables exceed the allocation limit set by "
                                               "odt_debug_set_table_alloc_limit");
        }
    }
    cudaError_t e = cudaGetDevice(&p->device);
    if (e != cudaSuccess) {
        delete p;
        return cuda_fail(e, "cudaGetDevice");
    }
    e = cudaMalloc(&p->d_tables, o);
    if (e != cudaSuccess) {
        delete p;
        return e == cudaErrorMemoryAllocation ? fail(ODT_ERR_OUT_OF_MEMORY, "cudaMalloc of plan tables failed")
                                              : cuda_fail(e, "cudaMalloc");
    }
    char *base = (char *)p->d_tables;
    struct Up { size_t off; const void *src; size_t n; } ups[] = {
        {oG, G.data(), K * 8}, {oW, W.data(), K * 8}, {oS, S.data(), K * 8}, {oA, AL.data(), 2 * K * 8},
        {oB, BE.data(), 2 * K * 8}, {oTx, twx.data(), (size_t)lNx * 8}, {oTy, twy.data(), (size_t)lNy * 8},
        {oZ, zp.data(), 2 * odt::ZPOW_N * 4}};
    for (const Up &u : ups) {
        e = cudaMemcpy(base + u.off, u.src, u.n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(p->d_tables);
            delete p;
            return cuda_fail(e, "cudaMemcpy of plan tables");
        }
    }
    e = cudaMemset(base + oSt, 0, 16);
    if (e != cudaSuccess) {
        cudaFree(p->d_tables);
        delete p;
        return cuda_fail(e, "cudaMemset");
    }
    p->tab.G = (const float2 *)(base + oG);
    p->tab.wsplit = (const float2 *)(base + oW);
    p->tab.step = (const float2 *)(base + oS);
    p->tab.alpha = (const float2 *)(base + oA);
    p->tab.beta = (const float2 *)(base + oB);
    p->tab.twx = (const float2 *)(base + oTx);
    p->tab.twy = (const float2 *)(base + oTy);
    p->tab.zpow = (const float *)(base + oZ);
    p->d_status = (int *)(base + oSt);

    // ---- batching: the largest angle batch (and column-stage chunk) whose
    // workspace fits the limit
    // tilted path, order >= 2: the column stage leaves the y-prefilter
    // terms to the row stage and stores each job's raw edge samples (4 np
    // rows) after the chunk's jobs
    p->jobs = 0;
    p->ydefer = 0;
    {
        const StageParams G = stage_params(p);
        p->ydefer = (tilted && pf && !odt::single_row_plan(G)) ? 1 : 0;
    }
    const size_t plane_row_bytes = (size_t)d.ny * lNx * 8;           // one job's column-stage output
    const size_t edge_row_bytes = p->ydefer ? (size_t)4 * np * lNx * 8 : 0;  // its y-prefilter edge samples
    // one angle's coefficient slab [z][x][ypitch] (the adjoint's slab
    // gradients [y][z][x] fit too)
    const size_t slab_bytes = (size_t)nz * odt::yaxis_slab_pitch(d.ny) * d.nx * 8;
    const size_t rowspec_bytes = (size_t)lNy * lNx * 8;              // one angle's row spectra
    const size_t tab_bytes = pf ? (size_t)2 * np * d.ny * lNx * 8 : 0;  // one angle's z-boundary rows
    const size_t vol_bytes = (size_t)nz * d.ny * d.nx * 8;           // compensation buffer
    const uint64_t limit = d.workspace_limit ? d.workspace_limit : kDefaultWorkspace;
    // chunk buffers take at most a quarter of the limit, so tight limits
    // (save_memory) keep room for a batch of angles
    const uint64_t plane_budget = std::min<uint64_t>(kPlaneBudget, limit / 4);
    // and at most 1024 planes (where the gain levels off), so small planes do
    // not take memory for nothing
    const size_t jobs_cap = std::max<size_t>(16, std::min<size_t>(1024, plane_budget / 2 / plane_row_bytes));
    auto layout = [&](int batch, size_t jobs, bool commit) -> size_t {
        const int nbatches = (d.num_angles + batch - 1) / batch;
        size_t w = 0;
        const size_t o_rowspec = w; w = align_up(w + (size_t)batch * rowspec_bytes);
        const size_t o_T = w; w = align_up(w + jobs * (plane_row_bytes + edge_row_bytes));
        const size_t o_T2 = w; w = align_up(w + jobs * (plane_row_bytes + edge_row_bytes));
        const size_t o_Tab = w; w = align_up(w + (size_t)batch * tab_bytes);
        const size_t o_slab = w; w = align_up(w + (size_t)batch * slab_bytes);
        const size_t o_comp = w; w = align_up(w + (nbatches > 1 ? vol_bytes : 0));
        const size_t o_rot = w;
        w = align_up(w + odt::rotate_scratch_bytes(batch, d.ny, d.nx, nz, tilted ? 1 : 0));
        if (commit) {
            p->batch = batch;
            p->jobs = (int)jobs;
            p->off_rowspec = o_rowspec;
            p->off_T = o_T;
            p->off_T2 = o_T2;
            p->off_Tab = o_Tab;
            p->off_slab = o_slab;
            p->off_comp = o_comp;
            p->off_rot = o_rot;
            p->ws_bytes = w;
        }
        return w;
    };
    auto jobs_for = [&](int batch) {
        size_t jobs = std::min((size_t)batch * nz, jobs_cap);
        return jobs >= 16 ? jobs / 16 * 16 : jobs;
    };
    int best = 0;
    for (int lo = 1, hi = d.num_angles; lo <= hi;) {  // ws grows with the batch
        const int mid = lo + (hi - lo) / 2;
        if (layout(mid, jobs_for(mid), false) <= limit) {
            best = mid;
            lo = mid + 1;
        } else {
            hi = mid - 1;
        }
    }
    // a single batch needs no compensation buffer, so it can fit when a
    // slightly smaller batch does not
    if (best < d.num_angles && layout(d.num_angles, jobs_for(d.num_angles), false) <= limit)
        best = d.num_angles;
    if (best > 0) {
        layout(best, jobs_for(best), true);
    } else {
        // one angle per batch; shrink the column-stage chunk toward the limit
        size_t jobs = jobs_for(1);
        while (jobs > 1 && layout(1, jobs, false) > limit)
            jobs = jobs > 16 ? jobs - 16 : jobs - 1;
        layout(1, jobs, true);
    }

    {
        const size_t spec_b = (size_t)p->batch * lNy * lNx * 8;
        size_t w = p->ws_bytes;
        p->off_Qg = w; w = align_up(w + spec_b);
        p->off_W = w; w = align_up(w + spec_b);
        p->off_Pg = w; w = align_up(w + spec_b);
        // the volume gradient in the [z][x][y] order (y-axis adjoint)
        p->off_vT = w; w = align_up(w + (size_t)nz * d.ny * d.nx * 8);
        p->adj_ws_bytes = w;
    }

    p->col_slots = 0;
    StageParams P = stage_params(p);
    e = odt::configure_kernels(P);
    if (e == cudaSuccess) {
        p->col_slots = odt::columns_slots(P);
        P.col_slots = p->col_slots;
    P.zshift = (float)d.z_shift;
    }
    if (e == cudaSuccess && !tilted)
        e = odt::configure_rotate_kernels();
    if (e == cudaSuccess)
        e = odt::configure_adjoint_kernels(P);
    if (e == cudaSuccess && !tilted)
        e = odt::configure_rotate_adjoint_kernels();
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&p->s2, cudaStreamNonBlocking);
    for (cudaEvent_t *ev : {&p->ev_fork, &p->ev_join, &p->ev_col[0], &p->ev_col[1], &p->ev_row[0], &p->ev_row[1]})
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        destroy_sync_objects(p);
        cudaFree(p->d_tables);
        delete p;
        return cuda_fail(e, "kernel configuration");
    }
    *out = p;
    return ODT_OK;
}

odt_status odt_bpp3d_workspace_size(const odt_bpp3d_plan *plan, uint64_t *bytes)
{
    if (!plan || !bytes)
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL argument");
    *bytes = plan->ws_bytes;
    return ODT_OK;
}

odt_status odt_bpp3d_angle_batch(const odt_bpp3d_plan *plan, int32_t *batch)
{
    if (!plan || !batch)
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL argument");
    *batch = plan->batch;
    return ODT_OK;
}

}  // extern "C"

namespace {

// Event pair around one launch, summed into a stage slot after the run.
struct LaunchTimer {
    odt_stage_timing *t;
    cudaStream_t s;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev;
    explicit LaunchTimer(odt_stage_timing *timing, cudaStream_t stream) : t(timing), s(stream) {}
    void begin(int stage)
    {
        if (!t)
            return;
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
        ev.push_back({stage, {a, b}});
    }
    void end(double bytes)
    {
        if (!t)
            return;
        cudaEventRecord(ev.back().second.second, s);
        t->launches[ev.back().first] += 1;
        t->bytes[ev.back().first] += bytes;
    }
    cudaError_t finish()
    {
        if (!t)
            return cudaSuccess;
        cudaError_t e = cudaStreamSynchronize(s);
        for (auto &x : ev) {
            float ms = 0.f;
            if (e == cudaSuccess)
                e = cudaEventElapsedTime(&ms, x.second.first, x.second.second);
            t->ms[x.first] += ms;
            cudaEventDestroy(x.second.first);
            cudaEventDestroy(x.second.second);
        }
        ev.clear();
        return e;
    }
};

odt_status run_plan(const odt_bpp3d_plan *plan, const void *sino, const double *weights, const double *geometry,
                    const float *gain, const void *again, void *volume, void *workspace, void *stream,
                    odt_stage_timing *timing)
{
    if (!plan || !sino || !geometry || !volume || (!workspace && plan->ws_bytes))
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL pointer argument");
    if (((uintptr_t)workspace % kAlign) != 0)
        return fail(ODT_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    const odt_status dst = check_device(plan);
    if (dst != ODT_OK)
        return dst;
    const odt_bpp3d_desc &d = plan->d;
    cudaStream_t s = (cudaStream_t)stream;
    StageParams P = stage_params(plan);
    P.gain = gain;
    const size_t spec_elems = (size_t)plan->d.pad_ny * plan->d.pad_nx;
    char *ws = (char *)workspace;
    float2 *rowspec = (float2 *)(ws + plan->off_rowspec);
    float2 *T = (float2 *)(ws + plan->off_T);
    float2 *Tab = (float2 *)(ws + plan->off_Tab);
    float2 *slab = (float2 *)(ws + plan->off_slab);
    float2 *comp = (float2 *)(ws + plan->off_comp);
    void *rot_scratch = ws + plan->off_rot;
    const size_t in_elem = d.input_dtype == ODT_INPUT_C128 ? 16 : 8;
    const int geo_stride = d.geometry == ODT_GEOM_AFFINE3D ? 12 : 6;
    const int nbatches = (d.num_angles + plan->batch - 1) / plan->batch;
    const double plane_in = (double)d.ny * d.nx, spec = (double)d.pad_ny * d.pad_nx;
    const double vol = (double)plan->nz * d.ny * d.nx;
    const double out_elem = d.onlyreal ? 4.0 : 8.0;
    if (timing)
        std::memset(timing, 0, sizeof(*timing));
    LaunchTimer lt(timing, s);
    cudaError_t e;
    for (int b = 0; b < nbatches; ++b) {
        const int a0 = b * plan->batch;
        const int nb = std::min(plan->batch, d.num_angles - a0);
        const char *sino_b = (const char *)sino + (size_t)a0 * d.ny * d.nx * in_elem;
        P.again = again ? (const float2 *)again + (size_t)a0 * spec_elems : nullptr;
        lt.begin(ODT_STAGE_ROWS_FORWARD);
        e = odt::launch_rows_forward(P, sino_b, weights ? weights + a0 : nullptr, nb, rowspec, s);
        if (e != cudaSuccess)
            return cuda_fail(e, "rows_forward launch");
        lt.end(nb * (plane_in * in_elem + spec * 8.0));
        if (d.intp_order >= 2) {
            lt.begin(ODT_STAGE_COLUMNS_PROPAGATE);
            e = odt::launch_columns_boundary(P, rowspec, Tab, nb, s);
            if (e != cudaSuccess)
                return cuda_fail(e, "columns_boundary launch");
            lt.end(0.0);
        }
        const int total = nb * plan->nz;
        if (odt::single_row_plan(P)) {
            // single-row planes: the column stage is the identity and runs
            // inside the row stage, one launch over the batch's jobs
            lt.begin(ODT_STAGE_ROWS_INVERSE);
            e = odt::launch_rows_line(P, rowspec, Tab, slab, 0, total, s);
            if (e != cudaSuccess)
                return cuda_fail(e, "rows_line launch");
            lt.end(nb * spec * 8.0 + (double)total * plane_in * 8.0);
        } else if (timing) {
            // per-stage timing: the stages one after the other on one stream
            for (int q0 = 0; q0 < total; q0 += plan->jobs) {
                const int qn = std::min(plan->jobs, total - q0);
                lt.begin(ODT_STAGE_COLUMNS_PROPAGATE);
                e = odt::launch_columns_propagate(P, rowspec, T, q0, qn, s);
                if (e != cudaSuccess)
                    return cuda_fail(e, "columns_propagate launch");
                lt.end((double)qn / plan->nz * spec * 8.0);
                lt.begin(ODT_STAGE_ROWS_INVERSE);
                e = odt::launch_rows_inverse(P, T, Tab, slab, q0, qn, s);
                if (e != cudaSuccess)
                    return cuda_fail(e, "rows_inverse launch");
                lt.end((double)qn * plane_in * 8.0);
            }
        } else {
            // chunk pipeline: columns(k) on s into buffer k%2 after rows(k-2)
            // released it; rows(k) on s2 after columns(k)
            float2 *Tb[2] = {T, (float2 *)(ws + plan->off_T2)};
            cudaStream_t s2 = plan->s2;
            if ((e = cudaEventRecord(plan->ev_fork, s)) || (e = cudaStreamWaitEvent(s2, plan->ev_fork, 0)))
                return cuda_fail(e, "stream fork");
            int k = 0;
            for (int q0 = 0; q0 < total; q0 += plan->jobs, ++k) {
                const int qn = std::min(plan->jobs, total - q0);
                const int buf = k & 1;
                if (k >= 2 && (e = cudaStreamWaitEvent(s, plan->ev_row[buf], 0)))
                    return cuda_fail(e, "stream wait");
                e = odt::launch_columns_propagate(P, rowspec, Tb[buf], q0, qn, s);
                if (e != cudaSuccess)
                    return cuda_fail(e, "columns_propagate launch");
                if ((e = cudaEventRecord(plan->ev_col[buf], s)) || (e = cudaStreamWaitEvent(s2, plan->ev_col[buf], 0)))
                    return cuda_fail(e, "stream order");
                e = odt::launch_rows_inverse(P, Tb[buf], Tab, slab, q0, qn, s2);
                if (e != cudaSuccess)
                    return cuda_fail(e, "rows_inverse launch");
                if ((e = cudaEventRecord(plan->ev_row[buf], s2)))
                    return cuda_fail(e, "stream order");
            }
            // join: everything after (the resampling, the next batch) waits
            // for the row stage
            if ((e = cudaEventRecord(plan->ev_join, s2)) || (e = cudaStreamWaitEvent(s, plan->ev_join, 0)))
                return cuda_fail(e, "stream join");
        }
        RotParams R;
        R.ny = d.ny;
        R.nx = d.nx;
        R.nz = plan->nz;
        R.ypitch = P.ypitch;
        R.nbatch_angles = nb;
        R.first_pass = b == 0;
        R.last_pass = b == nbatches - 1;
        R.onlyreal = d.onlyreal;
        R.status = plan->d_status;
        lt.begin(ODT_STAGE_ROTATE);
        e = odt::launch_rotate(R, d.intp_order, d.geometry == ODT_GEOM_AFFINE3D, slab,
                               geometry + (size_t)a0 * geo_stride, volume, comp, rot_scratch, s);
        if (e != cudaSuccess)
            return cuda_fail(e, "rotate launch");
        double rb = nb * vol * 8.0 + vol * out_elem;
        if (!R.first_pass)
            rb += vol * (out_elem + 8.0);
        if (!R.last_pass)
            rb += vol * 8.0;
        lt.end(rb);
    }
    e = lt.finish();
    if (e != cudaSuccess)
        return cuda_fail(e, "timing");
    return ODT_OK;
}

}  // namespace

extern "C" {

odt_status odt_bpp3d_execute(const odt_bpp3d_plan *plan, const void *sino, const double *weights,
                             const double *geometry, void *volume, void *workspace, void *stream)
{
    return run_plan(plan, sino, weights, geometry, nullptr, nullptr, volume, workspace, stream, nullptr);
}

odt_status odt_bpp3d_execute_gain(const odt_bpp3d_plan *plan, const void *sino, const double *weights,
                                  const double *geometry, const float *gain, const void *angle_gain,
                                  void *volume, void *workspace, void *stream)
{
    return run_plan(plan, sino, weights, geometry, gain, angle_gain, volume, workspace, stream, nullptr);
}

odt_status odt_bpp3d_adjoint_workspace_size(const odt_bpp3d_plan *plan, uint64_t *bytes)
{
    if (!plan || !bytes)
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (plan->d.intp_order > 3)
        return fail(ODT_ERR_UNSUPPORTED, "the adjoint is implemented for spline orders 0..3");
    *bytes = plan->adj_ws_bytes;
    return ODT_OK;
}

odt_status odt_bpp3d_adjoint(const odt_bpp3d_plan *plan, const void *sino, const double *weights,
                             const double *geometry, const float *gain, const void *angle_gain,
                             const void *vol_grad, void *sino_grad, float *gain_grad, void *angle_gain_grad,
                             void *workspace, void *stream)
{
    if (!plan || !geometry || !vol_grad || !workspace)
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL pointer argument");
    if (!sino_grad && !gain_grad && !angle_gain_grad)
        return ODT_OK;
    if ((gain_grad || angle_gain_grad) && !sino)
        return fail(ODT_ERR_INVALID_ARGUMENT, "the gain gradient needs the sinogram");
    if (((uintptr_t)workspace % kAlign) != 0)
        return fail(ODT_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    const odt_status dst = check_device(plan);
    if (dst != ODT_OK)
        return dst;
    const odt_bpp3d_desc &d = plan->d;
    const bool tilted = d.geometry == ODT_GEOM_AFFINE3D;
    const int geo_stride = tilted ? 12 : 6;
    if (d.onlyreal)
        return fail(ODT_ERR_UNSUPPORTED, "the adjoint needs a complex (onlyreal=0) plan");
    if (d.intp_order > 3)
        return fail(ODT_ERR_UNSUPPORTED, "the adjoint is implemented for spline orders 0..3");
    cudaStream_t s = (cudaStream_t)stream;
    StageParams P = stage_params(plan);
    P.gain = gain;
    char *ws = (char *)workspace;
    float2 *rowspec = (float2 *)(ws + plan->off_rowspec);
    float2 *T = (float2 *)(ws + plan->off_T);
    float2 *slab = (float2 *)(ws + plan->off_slab);
    float2 *Qg = (float2 *)(ws + plan->off_Qg);
    float2 *W = (float2 *)(ws + plan->off_W);
    float2 *Pg = (float2 *)(ws + plan->off_Pg);
    const size_t in_elem = d.input_dtype == ODT_INPUT_C128 ? 16 : 8;
    const size_t spec = (size_t)d.pad_ny * d.pad_nx;
    const int nbatches = (d.num_angles + plan->batch - 1) / plan->batch;
    cudaError_t e;
    const float2 *vg = (const float2 *)vol_grad;
    if (!tilted) {
        float2 *vT = (float2 *)(ws + plan->off_vT);
        e = odt::launch_volume_zxy(vg, vT, plan->nz, d.ny, d.nx, s);
        if (e != cudaSuccess)
            return cuda_fail(e, "volume transpose launch");
        vg = vT;
    }
    if (gain_grad) {
        e = cudaMemsetAsync(gain_grad, 0, spec * sizeof(float), s);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMemsetAsync");
    }
    for (int b = 0; b < nbatches; ++b) {
        const int a0 = b * plan->batch;
        const int nb = std::min(plan->batch, d.num_angles - a0);
        P.again = angle_gain ? (const float2 *)angle_gain + (size_t)a0 * spec : nullptr;
        RotParams R;
        R.ny = d.ny;
        R.nx = d.nx;
        R.nz = plan->nz;
        R.ypitch = P.ypitch;
        R.nbatch_angles = nb;
        R.first_pass = 1;
        R.last_pass = 1;
        R.onlyreal = 0;
        R.status = plan->d_status;
        e = odt::launch_rotate_adjoint(R, d.intp_order, tilted ? 1 : 0, vg,
                                       geometry + (size_t)a0 * geo_stride, slab, ws + plan->off_rot, s);
        if (e != cudaSuccess)
            return cuda_fail(e, "rotate_adjoint launch");
        if (gain_grad || angle_gain_grad) {
            const char *sino_b = (const char *)sino + (size_t)a0 * d.ny * d.nx * in_elem;
            e = odt::launch_rows_forward(P, sino_b, weights ? weights + a0 : nullptr, nb, rowspec, s);
            if (e != cudaSuccess)
                return cuda_fail(e, "rows_forward launch");
        }
        e = cudaMemsetAsync(Qg, 0, (size_t)nb * spec * sizeof(float2), s);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMemsetAsync");
        const int total = nb * plan->nz;
        for (int q0 = 0; q0 < total; q0 += plan->jobs) {
            const int qn = std::min(plan->jobs, total - q0);
            e = odt::launch_adj_rows(P, slab, T, q0, qn, s);
            if (e != cudaSuccess)
                return cuda_fail(e, "adj_rows launch");
            e = odt::launch_adj_columns(P, T, Qg, q0, qn, s);
            if (e != cudaSuccess)
                return cuda_fail(e, "adj_columns launch");
        }
        e = odt::launch_adj_spectrum(P, rowspec, Qg, gain_grad,
                                     angle_gain_grad ? (float2 *)angle_gain_grad + (size_t)a0 * spec : nullptr, W,
                                     nb, s);
        if (e != cudaSuccess)
            return cuda_fail(e, "adj_spectrum launch");
        if (sino_grad) {
            e = odt::launch_adj_rows_full(P, W, Pg, nb, s);
            if (e != cudaSuccess)
                return cuda_fail(e, "adj_rows_full launch");
            e = odt::launch_adj_pad(P, Pg, weights ? weights + a0 : nullptr, nb,
                                    (float2 *)sino_grad + (size_t)a0 * d.ny * d.nx, s);
            if (e != cudaSuccess)
                return cuda_fail(e, "adj_pad launch");
        }
    }
    return ODT_OK;
}

odt_status odt_bpp3d_execute_timed(const odt_bpp3d_plan *plan, const void *sino, const double *weights,
                                   const double *geometry, void *volume, void *workspace, void *stream,
                                   odt_stage_timing *timing)
{
    if (!timing)
        return fail(ODT_ERR_INVALID_ARGUMENT, "timing is NULL");
    return run_plan(plan, sino, weights, geometry, nullptr, nullptr, volume, workspace, stream, timing);
}

odt_status odt_bpp3d_launch_count(const odt_bpp3d_plan *plan, int64_t *launches)
{
    if (!plan || !launches)
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL argument");
    const int A = plan->d.num_angles;
    const int nbatches = (A + plan->batch - 1) / plan->batch;
    int64_t n = 0;
    for (int b = 0; b < nbatches; ++b) {
        const int nb = std::min(plan->batch, A - b * plan->batch);
        const int64_t total = (int64_t)nb * plan->nz;
        if (odt::single_row_plan(stage_params(plan)))
            n += 3;  // row spectra, fused column + row stage, resampling
        else
            n += 2 + 2 * ((total + plan->jobs - 1) / plan->jobs);
        if (plan->d.intp_order >= 2)
            n += 1;  // z-prefilter boundary columns
        if (plan->d.geometry == ODT_GEOM_Y_AXIS)
            n += 1;  // per-(angle, tile) geometry setup
    }
    *launches = n;
    return ODT_OK;
}

odt_status odt_bpp3d_read_status(const odt_bpp3d_plan *plan, void *stream)
{
    if (!plan)
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL plan");
    const odt_status dst = check_device(plan);
    if (dst != ODT_OK)
        return dst;
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, plan->d_status, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "status read");
    if (h != 0) {
        // cleared synchronously, so a failed clear is reported here and not
        // by some later call
        e = cudaMemset(plan->d_status, 0, sizeof(int));
        if (e != cudaSuccess)
            return cuda_fail(e, "status clear");
        char buf[96];
        snprintf(buf, sizeof buf, "device check failed (bits 0x%x)", h);
        return fail(ODT_ERR_DEVICE_CHECK, buf);
    }
    return ODT_OK;
}

odt_status odt_debug_inject_status(const odt_bpp3d_plan *plan, int32_t bits, void *stream)
{
    if (!plan)
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL plan");
    if (bits < 0 || bits > 255)
        return fail(ODT_ERR_INVALID_ARGUMENT, "status bits must be in 0..255");
    const odt_status dst = check_device(plan);
    if (dst != ODT_OK)
        return dst;
    // the word's low byte (little-endian), stream-ordered like a kernel's
    // report; the upper bytes are cleared
    cudaError_t e = cudaMemsetAsync(plan->d_status, 0, sizeof(int), (cudaStream_t)stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(plan->d_status, bits, 1, (cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "status injection");
    return ODT_OK;
}

odt_status odt_debug_set_table_alloc_limit(uint64_t bytes)
{
    std::lock_guard<std::mutex> lock(g_debug_mutex);
    g_table_alloc_limit = bytes;
    return ODT_OK;
}

odt_status odt_bpp3d_plan_destroy(odt_bpp3d_plan *plan)
{
    if (!plan)
        return ODT_OK;
    destroy_sync_objects(plan);
    cudaError_t e = cudaFree(plan->d_tables);
    delete plan;
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaFree");
    return ODT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Execution without allocation.
//
// Some callers cannot allocate device memory when they run a
// reconstruction: code inside a region where a cudaMalloc would stall the
// device or is not allowed (a latency-critical acquisition loop, a stream
// that is being captured, a framework that owns every byte of device
// memory and only hands out pointers to its own tensors).  For them the
// execution below takes its scratch space from a fixed array that is part of
// the library's device image instead of a caller-provided workspace.
//
// * The array is ODT_NOALLOC_SCRATCH_BYTES (64 MiB) per device; every device
//   on which the library's device code is loaded holds it until the process
//   exits.  Plans whose workspace is larger are rejected: create the plan
//   with desc.workspace_limit <= ODT_NOALLOC_SCRATCH_BYTES.
// * The first call on a device looks up the array's device address
//   (cudaGetSymbolAddress) with that device current, once; make that first
//   call before any stream capture.
// * Every call on a device uses the same array and leaves its contents
//   behind; nothing in it has to start at zero (each stage writes what the
//   next reads).  Calls whose executions overlap on the GPU race on it: run
//   them on one stream, or order them.
static __device__ __align__(256) unsigned char g_noalloc_scratch[ODT_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_addr[kMaxDevices];
}  // namespace

extern "C" odt_status odt_bpp3d_execute_noalloc(const odt_bpp3d_plan *plan, const void *sino,
                                                const double *weights, const double *geometry, void *volume,
                                                void *stream)
{
    if (!plan)
        return fail(ODT_ERR_INVALID_ARGUMENT, "NULL plan");
    if (plan->ws_bytes > ODT_NOALLOC_SCRATCH_BYTES) {
        char buf[200];
        snprintf(buf, sizeof buf,
                 "plan needs %llu bytes of scratch, the static scratch holds %llu; create the plan with "
                 "workspace_limit <= %llu",
                 (unsigned long long)plan->ws_bytes, (unsigned long long)ODT_NOALLOC_SCRATCH_BYTES,
                 (unsigned long long)ODT_NOALLOC_SCRATCH_BYTES);
        return fail(ODT_ERR_INVALID_ARGUMENT, buf);
    }
    // the scratch of the plan's device, which must be current
    const odt_status dst = check_device(plan);
    if (dst != ODT_OK)
        return dst;
    const int dev = plan->device;
    cudaError_t e = cudaSuccess;
    if (dev < 0 || dev >= kMaxDevices)
        return fail(ODT_ERR_UNSUPPORTED, "device ordinal beyond the static scratch table");
    void *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_addr[dev]) {
            e = cudaGetSymbolAddress(&g_noalloc_addr[dev], g_noalloc_scratch);
            if (e != cudaSuccess) {
                g_noalloc_addr[dev] = nullptr;
                return cuda_fail(e, "cudaGetSymbolAddress of the static scratch");
            }
        }
        scratch = g_noalloc_addr[dev];
    }
    return run_plan(plan, sino, weights, geometry, nullptr, nullptr, volume, scratch, stream, nullptr);
}
