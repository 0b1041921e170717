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
        k_odt_to_ri_complex<float><<<g, 256, 0, s>>>((const C2<float> *)f, (C2<float> *)ri, n, (float)inv,
                                                     (float)nm);
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
    if (dtype == ODT_DATA_F32 || dtype == ODT_DATA_C64)
        k_opt_to_ri<float><<<g, 256, 0, s>>>((const float *)f, (float *)ri, m, (float)twopi, (float)res, (float)nm,
                                             cplx);
    else
        k_opt_to_ri<double><<<g, 256, 0, s>>>((const double *)f, (double *)ri, m, twopi, res, nm, cplx);
    return launched("opt_to_ri");
}

}  // extern "C"
