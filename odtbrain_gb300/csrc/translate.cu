// Object function -> refractive index, elementwise on the GPU.
//
//   odt_to_ri (odtbrain/_translate_ri.py:5-57):  n = nm * sqrt(f / km^2 + 1),
//       km = 2 pi nm / res, the principal square root with a non-negative
//       real part (complex f), NaN where f / km^2 + 1 < 0 (real f);
//   opt_to_ri (odtbrain/_translate_ri.py:60-93):  n = nm + f / (2 pi) * res.
//
// FP32 for float32 / complex64 data, FP64 for float64 / complex128.  The
// complex square root is the half-angle form: for z = x + i y,
// t = sqrt((|x| + |z|) / 2); sqrt(z) = (t, y / (2t)) for x >= 0 and
// (|y| / (2t), copysign(t, y)) otherwise (no cancellation in either branch).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>

#include "../../include/odtbrain_gb300.h"
#include "odt_internal.cuh"

namespace odt {
namespace {

template <class T>
struct C2 {
    T x, y;
};

template <class T>
__device__ __forceinline__ C2<T> csqrt_principal(T x, T y)
{
    C2<T> r;
    if (x == T(0) && y == T(0)) {
        r.x = T(0);
        r.y = y;
        return r;
    }
    const T t = sqrt((fabs(x) + hypot(x, y)) * T(0.5));
    if (x >= T(0)) {
        r.x = t;
        r.y = y / (T(2) * t);
    } else {
        r.x = fabs(y) / (T(2) * t);
        r.y = copysign(t, y);
    }
    return r;
}

template <class T>
__global__ void k_odt_to_ri_complex(const C2<T> *f, C2<T> *ri, long long n, T inv_km2, T nm)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const C2<T> v = f[i];
        C2<T> s = csqrt_principal<T>(v.x * inv_km2 + T(1), v.y * inv_km2);
        s.x *= nm;
        s.y *= nm;
        if (s.x < T(0)) {
            s.x = -s.x;
            s.y = -s.y;
        }
        ri[i] = s;
    }
}

// complex64 with 16-byte aligned pointers: two elements per 16-byte access
// and two accesses in flight per thread (the arithmetic of each element is
// that of k_odt_to_ri_complex)
__device__ __forceinline__ float2 ri_c64(float x, float y, float inv_km2, float nm)
{
    C2<float> s = csqrt_principal<float>(x * inv_km2 + 1.f, y * inv_km2);
    s.x *= nm;
    s.y *= nm;
    if (s.x < 0.f) {
        s.x = -s.x;
        s.y = -s.y;
    }
    return make_float2(s.x, s.y);
}

__device__ __forceinline__ float4 ri_c64x2(float4 v, float inv_km2, float nm)
{
    const float2 a = ri_c64(v.x, v.y, inv_km2, nm), b = ri_c64(v.z, v.w, inv_km2, nm);
    return make_float4(a.x, a.y, b.x, b.y);
}

__global__ void k_odt_to_ri_c64x2(const float4 *f, float4 *ri, long long n2, float inv_km2, float nm)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + stride < n2; i += 2 * stride) {
        const float4 a = __ldcs(f + i), b = __ldcs(f + i + stride);
        __stcs(ri + i, ri_c64x2(a, inv_km2, nm));
        __stcs(ri + i + stride, ri_c64x2(b, inv_km2, nm));
    }
    if (i < n2)
        __stcs(ri + i, ri_c64x2(__ldcs(f + i), inv_km2, nm));
}

template <class T>
__global__ void k_odt_to_ri_real(const T *f, T *ri, long long n, T inv_km2, T nm)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        ri[i] = nm * sqrt(f[i] * inv_km2 + T(1));  // NaN below -1, like NumPy
}

template <class T>
__global__ void k_opt_to_ri(const T *f, T *ri, long long n, T twopi, T res, T nm, int cplx)
{
    // n elements of T, each (f / (2 pi)) * res in the reference's order; for
    // complex data only the real parts are shifted by nm
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const T v = (f[i] / twopi) * res;
        ri[i] = (!cplx || (i & 1) == 0) ? nm + v : v;
    }
}

// float32 / complex64 data with 16-byte aligned pointers: four floats per
// access, two accesses in flight per thread; element 4i is even, so for
// complex data the real parts are components x and z
__device__ __forceinline__ float4 opt_f32x4(float4 v, float twopi, float res, float nm, int cplx)
{
    float4 o = make_float4((v.x / twopi) * res, (v.y / twopi) * res, (v.z / twopi) * res, (v.w / twopi) * res);
    o.x += nm;
    o.z += nm;
    if (!cplx) {
        o.y += nm;
        o.w += nm;
    }
    return o;
}

__global__ void k_opt_to_ri_f32x4(const float4 *f, float4 *ri, long long n4, float twopi, float res, float nm,
                                  int cplx)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + stride < n4; i += 2 * stride) {
        const float4 a = __ldcs(f + i), b = __ldcs(f + i + stride);
        __stcs(ri + i, opt_f32x4(a, twopi, res, nm, cplx));
        __stcs(ri + i + stride, opt_f32x4(b, twopi, res, nm, cplx));
    }
    if (i < n4)
        __stcs(ri + i, opt_f32x4(__ldcs(f + i), twopi, res, nm, cplx));
}

bool aligned16(const void *a, const void *b)
{
    return ((uintptr_t)a % 16) == 0 && ((uintptr_t)b % 16) == 0;
}

unsigned grid_for(long long n)
{
    const long long g = (n + 255) / 256;
    return (unsigned)(g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16);
}

odt_status check_args(const void *f, const void *ri, int64_t n, int32_t dtype, double res, double nm)
{
    if (!f || !ri || n < 0)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "NULL pointer or negative count");
    if (dtype < ODT_DATA_F32 || dtype > ODT_DATA_C128)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "unknown data type");
    if (!(res > 0) || !(nm > 0))
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "res and nm must be positive");
    const size_t align = (dtype == ODT_DATA_F32) ? 4 : (dtype == ODT_DATA_C128 ? 16 : 8);
    if ((uintptr_t)f % align || (uintptr_t)ri % align)
        return (odt_status)set_error(ODT_ERR_INVALID_ARGUMENT, "misaligned data pointer");
    return ODT_OK;
}

odt_status launched(const char *what)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return (odt_status)set_error(ODT_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(e)).c_str());
    return ODT_OK;
}

}  // namespace
}  // namespace odt

using namespace odt;

extern "C" {

odt_status odt_odt_to_ri(const void *f, void *ri, int64_t n, int32_t dtype, double res, double nm, void *stream)
{
    const odt_status st = check_args(f, ri, n, dtype, res, nm);
    if (st != ODT_OK || n == 0)
        return st;
    const double km = (2.0 * M_PI * nm) / res;
    const double inv = 1.0 / (km * km);
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned g = grid_for(n);
    switch (dtype) {
    case ODT_DATA_F32:
        k_odt_to_ri_real<float><<<g, 256, 0, s>>>((const float *)f, (float *)ri, n, (float)inv, (float)nm);
        break;
    case ODT_DATA_F64:
        k_odt_to_ri_real<double><<<g, 256, 0, s>>>((const double *)f, (double *)ri, n, inv, nm);
        break;
    case ODT_DATA_C64:
        if (aligned16(f, ri) && n >= 2) {
            // pairs through 16-byte accesses, an odd last element alone
            const long long n2 = n / 2;
            k_odt_to_ri_c64x2<<<grid_for(n2), 256, 0, s>>>((const float4 *)f, (float4 *)ri, n2, (float)inv,
                                                            (float)nm);
            if (n % 2)
                k_odt_to_ri_complex<float><<<1, 32, 0, s>>>((const C2<float> *)f + (n - 1),
                                                            (C2<float> *)ri + (n - 1), 1, (float)inv, (float)nm);
        } else {
            k_odt_to_ri_complex<float><<<g, 256, 0, s>>>((const C2<float> *)f, (C2<float> *)ri, n, (float)inv,
                                                         (float)nm);
        }
        break;
    default:
        k_odt_to_ri_complex<double><<<g, 256, 0, s>>>((const C2<double> *)f, (C2<double> *)ri, n, inv, nm);
        break;
    }
    return launched("odt_to_ri");
}

odt_status odt_opt_to_ri(const void *f, void *ri, int64_t n, int32_t dtype, double res, double nm, void *stream)
{
    const odt_status st = check_args(f, ri, n, dtype, res, nm);
    if (st != ODT_OK || n == 0)
        return st;
    const double twopi = 2.0 * M_PI;
    cudaStream_t s = (cudaStream_t)stream;
    const int cplx = dtype == ODT_DATA_C64 || dtype == ODT_DATA_C128;
    const long long m = cplx ? 2 * n : n;
    const unsigned g = grid_for(m);
    if ((dtype == ODT_DATA_F32 || dtype == ODT_DATA_C64) && aligned16(f, ri) && m >= 4) {
        // quads through 16-byte accesses; the 0-3 floats left start at an
        // even index, so the real/imaginary pattern carries over
        const long long m4 = m / 4, done = 4 * m4;
        k_opt_to_ri_f32x4<<<grid_for(m4), 256, 0, s>>>((const float4 *)f, (float4 *)ri, m4, (float)twopi,
                                                        (float)res, (float)nm, cplx);
        if (m > done)
            k_opt_to_ri<float><<<1, 32, 0, s>>>((const float *)f + done, (float *)ri + done, m - done,
                                                (float)twopi, (float)res, (float)nm, cplx);
    } else if (dtype == ODT_DATA_F32 || dtype == ODT_DATA_C64) {
        k_opt_to_ri<float><<<g, 256, 0, s>>>((const float *)f, (float *)ri, m, (float)twopi, (float)res, (float)nm,
                                             cplx);
    } else
        k_opt_to_ri<double><<<g, 256, 0, s>>>((const double *)f, (double *)ri, m, twopi, res, nm, cplx);
    return launched("opt_to_ri");
}

}  // extern "C"
