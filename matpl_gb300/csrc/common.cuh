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

__host__ __device__ inline float __uint_as_float_hd(uint32_t b) {
    float f;
    memcpy(&f, &b, 4);
    return f;
}

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
// 64 x 64 -> 128-bit product.
__host__ __device__ inline void mul_u128(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
#ifdef __CUDA_ARCH__
    lo = a * b;
    hi = __umul64hi(a, b);
#else
    const unsigned __int128 p = (unsigned __int128)a * b;
    lo = (uint64_t)p;
    hi = (uint64_t)(p >> 64);
#endif
}

// Exact comparison of (K 2^ek)^2 with a positive normal double v (K < 2^58): -1, 0, +1 as
// the square is <, ==, > v.  Integer arithmetic only.
__host__ __device__ inline int cmp_square(uint64_t K, int ek, uint64_t v_bits) {
    const uint64_t D = (v_bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int dv = (int)((v_bits >> 52) & 0x7FF) - 1023 - 52;
    uint64_t ahi, alo;
    mul_u128(K, K, ahi, alo);                   // K^2 2^(2 ek)  vs  D 2^dv
    const int sh = dv - 2 * ek;                  // compare K^2 with D 2^sh
    uint64_t bhi = 0, blo = D;
    if (sh <= -64) {
        blo = 0;
    } else if (sh < 0) {
        blo = D >> (-sh);
        if ((blo << (-sh)) != D) {               // D 2^sh is not an integer: compare K^2 2^-sh
            const uint64_t chi = (ahi << (-sh)) | (-sh ? alo >> (64 + sh) : 0);
            const uint64_t clo = alo << (-sh);
            if (ahi >> (64 + sh)) return 1;      // K^2 2^-sh overflows 128 bits: larger
            return chi != 0 || clo > D ? 1 : (clo < D ? -1 : 0);
        }
    } else if (sh >= 75) {
        return -1;                               // D 2^sh >= 2^127 > K^2 (K < 2^58... 2^116)
    } else if (sh >= 64) {
        bhi = D << (sh - 64);
        blo = 0;
    } else if (sh > 0) {
        bhi = D >> (64 - sh);
        blo = D << sh;
    }
    if (ahi != bhi) return ahi < bhi ? -1 : 1;
    return alo < blo ? -1 : (alo > blo ? 1 : 0);
}

// The float of the correctly rounded double sqrt of a positive normal double v, i.e.
// (float)sqrt_rn(v) bit for bit, without the FP64 pipe.  From a single-precision estimate:
// (1) the float nearest to sqrt(v), by exact comparisons of v with the squares of the float
// midpoints on either side of it; (2) the double rounding of the reference (sqrt rounded to
// double, then to float): when sqrt_rn(v) falls exactly on a float midpoint m, that is when v
// lies within the squares of m -+ half a double ulp, the result is the even neighbour of m.
__host__ __device__ inline float sqrt_to_f32_bits(float estimate, uint64_t v_bits) {
    uint32_t yb;
    memcpy(&yb, &estimate, 4);
    for (int it = 0; it < 3; ++it) {
        const uint64_t Y = (yb & 0x7FFFFFu) | 0x800000u;
        const int ey = (int)((yb >> 23) & 0xFF) - 127 - 23;
        const int up = cmp_square(2 * Y + 1, ey - 1, v_bits);            // midpoint above y
        if (up < 0) { ++yb; continue; }
        if (up == 0) { if (Y & 1) ++yb; return __uint_as_float_hd(yb); }   // exact tie
        const bool pow2 = Y == 0x800000u;                                  // ulp below is half
        const int dn = pow2 ? cmp_square(4 * Y - 1, ey - 2, v_bits)
                            : cmp_square(2 * Y - 1, ey - 1, v_bits);      // midpoint below y
        if (dn > 0) { --yb; continue; }
        if (dn == 0) { if (Y & 1) --yb; return __uint_as_float_hd(yb); }
        break;
    }
    // (2) midpoints written with 54-bit odd numerators: m -+ u/2 = (M 2^(s+1) -+ 1) 2^(e-s-1),
    // M 2^e the midpoint (M odd, < 2^26) and u = 2^(e-s) its double ulp
    const uint64_t Y = (yb & 0x7FFFFFu) | 0x800000u;
    const int ey = (int)((yb >> 23) & 0xFF) - 127 - 23;
    {   // midpoint above y, M = 2Y + 1 (25 bits): s = 28
        const uint64_t K = ((2 * Y + 1) << 29) - 1;
        if (cmp_square(K, ey - 1 - 29, v_bits) <= 0) {          // sqrt_rn(v) = m
            if (Y & 1) ++yb;
            return __uint_as_float_hd(yb);
        }
    }
    {   // midpoint below y
        const bool pow2 = Y == 0x800000u;
        const uint64_t M = pow2 ? 4 * Y - 1 : 2 * Y - 1;        // 25 bits (26 for pow2... 25)
        const int e = pow2 ? ey - 2 : ey - 1;
        const uint64_t K = (M << 29) + 1;
        if (cmp_square(K, e - 29, v_bits) >= 0) {
            if (Y & 1) --yb;
            return __uint_as_float_hd(yb);
        }
    }
    return __uint_as_float_hd(yb);
}

template <typename TO> __device__ __forceinline__ TO conv(double v);
template <> __device__ __forceinline__ float conv<float>(double v) { return to_f32(v); }
template <> __device__ __forceinline__ double conv<double>(double v) { return v; }

// r = sqrt(dd) of a pair, in the output dtype: f64 correctly rounded; f32 the float nearest to
// that f64 value, formed without the FP64 pipe (sqrt_to_f32_bits).
template <typename TO> __device__ __forceinline__ TO pair_r(double dd);
template <> __device__ __forceinline__ double pair_r<double>(double dd) { return __dsqrt_rn(dd); }
template <> __device__ __forceinline__ float pair_r<float>(double dd) {
    return sqrt_to_f32_bits(sqrtf(to_f32(dd)), (unsigned long long)__double_as_longlong(dd));
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
