// Shared helpers for the matpl_gb300 kernels (sm_103a only).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <string>
#include "../../include/matpl_gb300.h"

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ < 1000)
#error "matpl_gb300 is built for sm_103a (GB300) only"
#endif

namespace matpl {

void set_error(const std::string &msg);

#define MATPL_REQUIRE(cond, code, msg)                 \
    do {                                               \
        if (!(cond)) {                                 \
            ::matpl::set_error(msg);                   \
            return (code);                             \
        }                                              \
    } while (0)

inline int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string(what) + ": " + cudaGetErrorString(e));
        return MATPL_ERR_CUDA;
    }
    return MATPL_OK;
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// The kernels of an entry point launch on the current device.  A device pointer that lives on
// another GPU would be read through peer mappings at best (an illegal address without peer
// access), so every entry point checks one of its device arrays here: MATPL_ERR_INVALID when
// it belongs to a device other than the current one.  Host, managed and unregistered memory
// pass (the LAMMPS path reads host arrays in place where the GPU can).
int require_current_device(const void *p, const char *what);

#define MATPL_REQUIRE_ON_DEVICE(p, what)                                        \
    do {                                                                        \
        const int matpl_dev_rc_ = ::matpl::require_current_device((p), (what)); \
        if (matpl_dev_rc_ != MATPL_OK) return matpl_dev_rc_;                    \
    } while (0)

// Optional per-kernel timing (matpl_profile_begin / matpl_profile_collect): when enabled,
// every launch site records a CUDA event pair on its own stream.
bool profiling_enabled();
void profile_record(const char *name, cudaEvent_t start, cudaEvent_t stop);
cudaEvent_t profile_event();

struct ProfScope {
    const char *name;
    cudaStream_t stream;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(const char *n, cudaStream_t s) : name(n), stream(s) {
        if (profiling_enabled()) {
            a = profile_event();
            b = profile_event();
            if (a && b) cudaEventRecord(a, stream);
        }
    }
    ~ProfScope() {
        if (a && b) {
            cudaEventRecord(b, stream);
            profile_record(name, a, b);
        }
    }
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Streaming multiprocessors of the current device (queried once per device; grids are sized
// in multiples of it).
int device_sms();

// Device math wrappers: the plain forms call CUDA's tanhf / tanh.
__device__ __forceinline__ float dev_tanh(float x) { return tanhf(x); }
__device__ __forceinline__ double dev_tanh(double x) { return tanh(x); }

// f64 -> f32 round-to-nearest-even in integer arithmetic (keeps the conversions off the FP64
// pipe, which runs 2 lanes per clock per SM on this part); magnitudes below the f32 normal
// range take the hardware conversion (never met by interatomic distances in Angstrom).
__device__ __forceinline__ float to_f32(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned ex = (hi >> 20) & 0x7ffu;
    const int e = (int)ex - 1023 + 127;
    if ((b << 1) == 0ull) return __uint_as_float(hi & 0x80000000u);     // signed zero
    if (e <= 0 || e >= 255) return __double2float_rn(v);
    const unsigned sign = hi & 0x80000000u;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    unsigned r = ((unsigned)e << 23) | m;
    r += (rest > 0x10000000u) || (rest == 0x10000000u && (m & 1u));
    return __uint_as_float(sign | r);
}
// Order-preserving integer key of a double (for exact comparisons outside the FP64 pipe).
__host__ __device__ inline long long dkey(double x) {
    long long b;
    memcpy(&b, &x, 8);
    return b >= 0 ? b : (long long)((unsigned long long)b ^ 0x7FFFFFFFFFFFFFFFull);
}

__host__ __device__ inline double dfrom(unsigned long long b) {
    double x;
    memcpy(&x, &b, 8);
    return x;
}

__host__ __device__ inline float dfrom_f(uint32_t b) {
    float x;
    memcpy(&x, &b, 4);
    return x;
}

// The float of the correctly rounded double square root of a positive normal double v, i.e.
// (float)sqrt_rn(v) bit for bit, with four FP64 operations instead of a double square root.
// y = sqrtf((float)v) is within one float ulp of sqrt(v), so the answer is y or a neighbour,
// decided by where s = sqrt_rn(v) lies relative to the float midpoints m = y -+ ulp/2 (exact
// doubles; in the bit pattern of double(y) they are -+ 2^28, across a power of two too).  With
// r = v - m*m (both operations exact: m*m has 50 bits and v, m*m are within a factor 2) and
// T = m * ulp64(m): s > m iff r > T, and s = m iff -T < r <= T (the doubles between the
// square roots of v's neighbours do not resolve the u64^2/4 term), the round-half-even cases
// of the double rounding included.
__host__ __device__ inline float sqrt_to_f32(float y, double v) {
    uint32_t fb;
    memcpy(&fb, &y, 4);
    // bit pattern of double(y) (y positive and normal), built without a conversion instruction
    const unsigned long long yb = ((unsigned long long)(((fb >> 23) & 0xFFu) + (1023u - 127u)) << 52) |
                                  ((unsigned long long)(fb & 0x7FFFFFu) << 29);
    const unsigned long long half = 1ull << 28;        // half a float ulp, in double units
    for (int side = 0; side < 2; ++side) {
        const unsigned long long mb = side == 0 ? yb + half : yb - half;
        const double m = dfrom(mb);
        const double r = v - m * m;                     // exact
        const long long em = (long long)((mb >> 52) & 0x7FF) - 1023;
        const double T = dfrom(mb + ((unsigned long long)(em - 52) << 52));   // m * ulp64(m)
        unsigned long long tb;
        memcpy(&tb, &T, 8);
        const long long kr = dkey(r), kT = (long long)tb;
        const long long kmT = (long long)((tb | (1ull << 63)) ^ 0x7FFFFFFFFFFFFFFFull);   // key of -T
        if (side == 0) {
            if (kr > kT) return dfrom_f(fb + 1);                   // s above m: round up
            if (kr > kmT) return dfrom_f((fb & 1u) ? fb + 1 : fb);  // s = m: to even
        } else {
            if (kr <= kmT) return dfrom_f(fb - 1);                 // s below m: round down
            if (kr <= kT) return dfrom_f((fb & 1u) ? fb - 1 : fb);  // s = m: to even
        }
    }
    return y;
}

template <typename TO> __device__ __forceinline__ TO conv(double v);
template <> __device__ __forceinline__ float conv<float>(double v) { return to_f32(v); }
template <> __device__ __forceinline__ double conv<double>(double v) { return v; }

// r = sqrt(dd) of a pair, in the output dtype: f64 correctly rounded; f32 the float nearest to
// that f64 value, formed with four FP64 operations (sqrt_to_f32).
template <typename TO> __device__ __forceinline__ TO pair_r(double dd);
template <> __device__ __forceinline__ double pair_r<double>(double dd) { return __dsqrt_rn(dd); }
template <> __device__ __forceinline__ float pair_r<float>(double dd) {
    return sqrt_to_f32(sqrtf(to_f32(dd)), dd);
}

// bit pattern of a non-negative double: orders like the value (NaN above +inf)
__device__ __forceinline__ unsigned long long ubits(double v) {
    return (unsigned long long)__double_as_longlong(v);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace matpl
