/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle for odtbrain_gb300.
 *
 * A plain-C FP64 restatement of the B-spline resampling that ODTbrain's 3D
 * backpropagation delegates to scipy.ndimage:
 *
 *   - odtbrain/_alg3d_bpp.py:68-81   (_rotate -> scipy.ndimage.rotate,
 *                                     axes=(0,2), reshape=False,
 *                                     mode="constant", cval=0)
 *   - odtbrain/_alg3d_bppt.py:931-944 (scipy.ndimage.affine_transform,
 *                                     mode="constant", cval=0)
 *
 * scipy.ndimage's C core is a third-party dependency of the reference
 * (pinned scipy>=1.4,<2 in pyproject.toml:32-37).  Its behaviour is restated
 * here from the published algorithms and from black-box measurements of the
 * installed scipy (1.18.1), which the CPU test-suite re-checks:
 *
 *   1. Prefilter: recursive B-spline filter with mirror ("whole-sample
 *      symmetric") boundaries along every axis (Unser, Aldroubi & Eden,
 *      "B-spline signal processing I/II", IEEE TSP 1993; Unser, "Splines:
 *      a perfect fit for signal and image processing", IEEE SPM 1999).
 *      mode="constant" prefilters exactly like mode="mirror".
 *   2. Coordinates: in_i = ((off_i + m_i0*o_0) + m_i1*o_1) [+ m_i2*o_2],
 *      every product rounded separately (this order reproduces scipy's
 *      out-of-domain decisions bit for bit; other orders do not).
 *   3. A sample whose coordinate lies outside [0, n-1] on any axis is cval=0.
 *   4. Inside, taps that fall outside [0, n-1] read mirror-extended
 *      coefficients.
 *   5. Tap start: floor(x+0.5) - order/2 for even orders, floor(x) - order/2
 *      for odd orders; weights are the centred B-spline of that order.
 *
 * Build: see oracle/build.py (gcc -O2 -fopenmp -ffp-contract=off).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- poles -- */
static int spline_poles(int order, double *z)
{
    switch (order) {
    case 2:
        z[0] = sqrt(8.0) - 3.0;
        return 1;
    case 3:
        z[0] = sqrt(3.0) - 2.0;
        return 1;
    case 4:
        z[0] = sqrt(664.0 - sqrt(438976.0)) + sqrt(304.0) - 19.0;
        z[1] = sqrt(664.0 + sqrt(438976.0)) - sqrt(304.0) - 19.0;
        return 2;
    case 5:
        z[0] = sqrt(67.5 - sqrt(4436.25)) + sqrt(26.25) - 6.5;
        z[1] = sqrt(67.5 + sqrt(4436.25)) - sqrt(26.25) - 6.5;
        return 2;
    default:
        return 0;
    }
}

/* Causal initial value for a mirror-extended line (period 2n-2), summed
 * exactly over one period. */
static double init_causal_mirror(const double *c, long n, long st, double z)
{
    double zn1 = pow(z, (double)(n - 1));
    double acc = c[0] + zn1 * c[(n - 1) * st];
    double zi = z;
    for (long i = 1; i < n - 1; ++i) {
        acc += zi * (c[i * st] + zn1 * c[(n - 1 - i) * st]);
        zi *= z;
    }
    return acc / (1.0 - zn1 * zn1);
}

/* Anti-causal initial value for the mirror extension. */
static double init_anticausal_mirror(const double *c, long n, long st,
                                     double z)
{
    return (z / (z * z - 1.0)) * (c[(n - 1) * st] + z * c[(n - 2) * st]);
}

/* In-place prefilter of one strided line. */
void odto_prefilter_line(double *c, long n, long st, int order)
{
    double z[2];
    int np = spline_poles(order, z);
    if (np == 0 || n < 2)
        return;
    double gain = 1.0;
    for (int k = 0; k < np; ++k)
        gain *= (1.0 - z[k]) * (1.0 - 1.0 / z[k]);
    for (long i = 0; i < n; ++i)
        c[i * st] *= gain;
    for (int k = 0; k < np; ++k) {
        double zk = z[k];
        c[0] = init_causal_mirror(c, n, st, zk);
        for (long i = 1; i < n; ++i)
            c[i * st] += zk * c[(i - 1) * st];
        c[(n - 1) * st] = init_anticausal_mirror(c, n, st, zk);
        for (long i = n - 2; i >= 0; --i)
            c[i * st] = zk * (c[(i + 1) * st] - c[i * st]);
    }
}

/* ------------------------------------------------------------- weights -- */
static inline long mirror_index(long i, long n)
{
    if (n == 1)
        return 0;
    long p = 2 * n - 2;
    if (i < 0)
        i = -i;
    i %= p;
    return i < n ? i : p - i;
}

/* Centred B-spline of degree n at x:
 * beta_n(x) = 1/n! * sum_k (-1)^k C(n+1,k) (x + (n+1)/2 - k)_+^n */
static double bspline_value(double x, int n)
{
    double acc = 0.0, binom = 1.0, fact = 1.0;
    for (int i = 2; i <= n; ++i)
        fact *= (double)i;
    for (int k = 0; k <= n + 1; ++k) {
        double u = x + 0.5 * (double)(n + 1) - (double)k;
        if (u > 0.0) {
            double p = 1.0;
            for (int i = 0; i < n; ++i)
                p *= u;
            acc += ((k & 1) ? -binom : binom) * p;
        }
        binom = binom * (double)(n + 1 - k) / (double)(k + 1);
    }
    return acc / fact;
}

/* Returns the first tap index and fills w[0..order]. */
static inline long spline_weights(double x, int order, double *w)
{
    long s;
    double t;
    switch (order) {
    case 0:
        s = (long)floor(x + 0.5);
        w[0] = 1.0;
        return s;
    case 1:
        s = (long)floor(x);
        t = x - (double)s;
        w[0] = 1.0 - t;
        w[1] = t;
        return s;
    case 2:
        s = (long)floor(x + 0.5);
        t = x - (double)s;
        w[0] = 0.5 * (0.5 - t) * (0.5 - t);
        w[1] = 0.75 - t * t;
        w[2] = 0.5 * (0.5 + t) * (0.5 + t);
        return s - 1;
    case 3: {
        s = (long)floor(x);
        t = x - (double)s;
        double u = 1.0 - t;
        w[0] = u * u * u / 6.0;
        w[1] = (4.0 - 6.0 * t * t + 3.0 * t * t * t) / 6.0;
        w[2] = (1.0 + 3.0 * t + 3.0 * t * t - 3.0 * t * t * t) / 6.0;
        w[3] = t * t * t / 6.0;
        return s - 1;
    }
    case 4:
    case 5: {
        /* general centred B-spline via truncated powers (de Boor) */
        if (order == 4)
            s = (long)floor(x + 0.5) - 2;
        else
            s = (long)floor(x) - 2;
        for (int k = 0; k <= order; ++k)
            w[k] = bspline_value(x - (double)(s + k), order);
        return s;
    }
    }
    return 0;
}

/* ----------------------------------------------------- 2D plane rotate -- */
static void prefilter_plane(double *p, long n0, long n1, int order)
{
    if (order < 2)
        return;
    for (long i = 0; i < n0; ++i)
        odto_prefilter_line(p + i * n1, n1, 1, order);
    for (long j = 0; j < n1; ++j)
        odto_prefilter_line(p + j, n0, n1, order);
}

static double interp2(const double *coef, long n0, long n1, const double *M,
                      const double *off, int order, long o0, long o1)
{
    double x0 = off[0];
    x0 += M[0] * (double)o0;
    x0 += M[1] * (double)o1;
    double x1 = off[1];
    x1 += M[2] * (double)o0;
    x1 += M[3] * (double)o1;
    if (x0 < 0.0 || x0 > (double)(n0 - 1) || x1 < 0.0 || x1 > (double)(n1 - 1))
        return 0.0;
    double w0[6], w1[6];
    long s0 = spline_weights(x0, order, w0);
    long s1 = spline_weights(x1, order, w1);
    long idx1[6];
    for (int j = 0; j <= order; ++j)
        idx1[j] = mirror_index(s1 + j, n1);
    double acc = 0.0;
    for (int i = 0; i <= order; ++i) {
        const double *row = coef + mirror_index(s0 + i, n0) * n1;
        double r = 0.0;
        for (int j = 0; j <= order; ++j)
            r += w1[j] * row[idx1[j]];
        acc += w0[i] * r;
    }
    return acc;
}

/*
 * vol[oz][y][ox] += rotate(slab[:, y, :]) for every y, where slab and vol
 * are real FP64 arrays of shape (nz, ny, nx) in C order.  M (2x2, row-major)
 * and off (2) map an output (oz, ox) to the input (iz, ix), as built by
 * scipy.ndimage.rotate for axes=(0, 2).
 */
int odto_rotate_y_acc(const double *slab, double *vol, long nz, long ny,
                      long nx, const double *M, const double *off, int order,
                      int nthreads)
{
    if (order < 0 || order > 5)
        return 1;
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        double *plane = (double *)malloc(sizeof(double) * nz * nx);
#ifdef _OPENMP
#pragma omp for schedule(dynamic)
#endif
        for (long y = 0; y < ny; ++y) {
            for (long z = 0; z < nz; ++z)
                for (long x = 0; x < nx; ++x)
                    plane[z * nx + x] = slab[(z * ny + y) * nx + x];
            prefilter_plane(plane, nz, nx, order);
            for (long oz = 0; oz < nz; ++oz)
                for (long ox = 0; ox < nx; ++ox)
                    vol[(oz * ny + y) * nx + ox] +=
                        interp2(plane, nz, nx, M, off, order, oz, ox);
        }
        free(plane);
    }
    return 0;
}

/* ---------------------------------------------------------- 3D affine -- */
static void prefilter_volume(double *v, long n0, long n1, long n2, int order,
                             int nthreads)
{
    if (order < 2)
        return;
    (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long i = 0; i < n0 * n1; ++i)
        odto_prefilter_line(v + i * n2, n2, 1, order);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long i = 0; i < n0 * n2; ++i) {
        long a = i / n2, c = i % n2;
        odto_prefilter_line(v + a * n1 * n2 + c, n1, n2, order);
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long i = 0; i < n1 * n2; ++i)
        odto_prefilter_line(v + i, n0, n1 * n2, order);
}

/*
 * out += affine_transform(in, M, off, order, mode="constant", cval=0) for a
 * real FP64 volume of shape (n0, n1, n2), C order; M is 3x3 row-major.
 * `work` must hold n0*n1*n2 doubles (the prefiltered coefficients).
 */
int odto_affine3d_acc(const double *in, double *out, double *work, long n0,
                      long n1, long n2, const double *M, const double *off,
                      int order, int nthreads)
{
    if (order < 0 || order > 5)
        return 1;
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#endif
    memcpy(work, in, sizeof(double) * n0 * n1 * n2);
    prefilter_volume(work, n0, n1, n2, order, nthreads);
    const long n[3] = {n0, n1, n2};
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic)
#endif
    for (long o0 = 0; o0 < n0; ++o0) {
        for (long o1 = 0; o1 < n1; ++o1) {
            for (long o2 = 0; o2 < n2; ++o2) {
                double x[3];
                int inside = 1;
                for (int i = 0; i < 3; ++i) {
                    double t = off[i];
                    t += M[3 * i + 0] * (double)o0;
                    t += M[3 * i + 1] * (double)o1;
                    t += M[3 * i + 2] * (double)o2;
                    x[i] = t;
                    if (t < 0.0 || t > (double)(n[i] - 1))
                        inside = 0;
                }
                if (!inside)
                    continue;
                double w[3][6];
                long s[3];
                for (int i = 0; i < 3; ++i)
                    s[i] = spline_weights(x[i], order, w[i]);
                long i2[6];
                for (int k = 0; k <= order; ++k)
                    i2[k] = mirror_index(s[2] + k, n2);
                double acc = 0.0;
                for (int a = 0; a <= order; ++a) {
                    long ia = mirror_index(s[0] + a, n0);
                    double ra = 0.0;
                    for (int b = 0; b <= order; ++b) {
                        const double *row =
                            work + (ia * n1 + mirror_index(s[1] + b, n1)) * n2;
                        double rb = 0.0;
                        for (int k = 0; k <= order; ++k)
                            rb += w[2][k] * row[i2[k]];
                        ra += w[1][b] * rb;
                    }
                    acc += w[0][a] * ra;
                }
                out[(o0 * n1 + o1) * n2 + o2] += acc;
            }
        }
    }
    return 0;
}
