// ##################################################################
//
// softdiv.cuh -- correctly rounded FP64 division on the integer pipes
//
// GB300 issues one FP64 warp instruction per ~70-80 cycles per SM
// sub-partition, and an IEEE division takes several of them; the
// integer units sit idle in the FP64-bound kernels.  These functions
// divide binary64 numbers with integer arithmetic only (plus one FP32
// division for a seed), giving the round-to-nearest-even quotient, i.e.
// exactly what the `/` operator gives, for normal operands.  Anything
// else (zero, subnormal, infinite or NaN divisor; infinite or NaN
// dividend; subnormal quotient) falls back to `/`.
//
// Method (Moller & Granlund, "Improved division by invariant integers",
// IEEE Trans. Computers 60(2), 2011): the divisor's 53-bit significand,
// shifted to a 64-bit word d, gets the reciprocal v = floor((2^128-1)/d)
// - 2^64 (their Algorithm 2); a 128-by-64-bit division with that
// reciprocal (their Algorithm 4) then yields the exact integer quotient
// and remainder of the dividend's significand scaled by 2^54 or 2^55,
// from which the rounded significand follows.  One reciprocal serves
// every division by the same divisor.
// ##################################################################
#ifndef HAMSTR_GPU_SOFTDIV_CUH
#define HAMSTR_GPU_SOFTDIV_CUH

#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace hamstr {
namespace sd {

__host__ __device__ __forceinline__ uint64_t mulhi(uint64_t a, uint64_t b)
{
#ifdef __CUDA_ARCH__
   return __umul64hi(a, b);
#else
   return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

__host__ __device__ __forceinline__ uint64_t bits(double x)
{
#ifdef __CUDA_ARCH__
   return (uint64_t)__double_as_longlong(x);
#else
   uint64_t u;
   std::memcpy(&u, &x, 8);
   return u;
#endif
}

__host__ __device__ __forceinline__ double from_bits(uint64_t u)
{
#ifdef __CUDA_ARCH__
   return __longlong_as_double((long long)u);
#else
   double x;
   std::memcpy(&x, &u, 8);
   return x;
#endif
}

// v = floor((2^128 - 1) / d) - 2^64 for 2^63 <= d < 2^64 (Algorithm 2 of
// Moller & Granlund; v0 = floor((2^19 - 3*2^8) / d9) from a correctly
// rounded FP32 division: the true quotient is never within 1/d9 > 2^-13
// below an integer, so the floor of the rounded quotient is exact)
__host__ __device__ __forceinline__ uint64_t reciprocal_word(uint64_t d)
{
   const uint64_t d0 = d & 1;
   const uint64_t d9 = d >> 55;
   const uint64_t d40 = (d >> 24) + 1;
   const uint64_t d63 = (d >> 1) + d0;
#ifdef __CUDA_ARCH__
   const uint64_t v0 = (uint64_t)__float2uint_rz(__fdiv_rn(523520.0f, (float)(uint32_t)d9));
#else
   const uint64_t v0 = (uint64_t)(523520u / (uint32_t)d9);
#endif
   const uint64_t v1 = (v0 << 11) - ((v0 * v0 * d40) >> 40) - 1;
   const uint64_t v2 = (v1 << 13) + ((v1 * ((1ull << 60) - v1 * d40)) >> 47);
   const uint64_t e = ((v2 >> 1) & (0 - d0)) - v2 * d63;
   const uint64_t v3 = (mulhi(v2, e) >> 1) + (v2 << 31);
   // v4 = v3 - floor((v3 + 2^64 + 1) d / 2^64)
   const uint64_t lo = v3 * d, hi = mulhi(v3, d);
   const uint64_t lo2 = lo + d;
   const uint64_t hi2 = hi + d + (lo2 < lo ? 1 : 0);
   return v3 - hi2;
}

// exact floor((u1 * 2^64 + u0) / d) and remainder, u1 < d, v = reciprocal_word(d)
// (Algorithm 4 of Moller & Granlund)
__host__ __device__ __forceinline__ uint64_t div_2by1(uint64_t u1, uint64_t u0, uint64_t d, uint64_t v, uint64_t& r)
{
   uint64_t q0 = v * u1;
   uint64_t q1 = mulhi(v, u1);
   const uint64_t t = q0 + u0;
   q1 = q1 + u1 + (t < q0 ? 1 : 0);
   q0 = t;
   q1 = q1 + 1;
   r = u0 - q1 * d;
   if (r > q0) {
      q1 = q1 - 1;
      r = r + d;
   }
   if (r >= d) {
      q1 = q1 + 1;
      r = r - d;
   }
   return q1;
}

// a divisor prepared once for several divisions
struct Divisor {
   double b;
   uint64_t d, v;    // significand << 11, its reciprocal word
   int eb;           // biased exponent
   uint64_t sign;
   bool ok;          // normal and finite: the integer path applies
};

__host__ __device__ __forceinline__ Divisor divisor(double b)
{
   Divisor D;
   const uint64_t B = bits(b);
   D.b = b;
   D.eb = (int)((B >> 52) & 0x7FF);
   D.sign = B & 0x8000000000000000ull;
   D.ok = D.eb != 0 && D.eb != 0x7FF;
   D.d = ((B & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) << 11;
   D.v = D.ok ? reciprocal_word(D.d) : 0;
   return D;
}

// the operands the integer path leaves to the `/` operator; kept out of
// line so that the many inlined divisions of a kernel share one copy of the
// hardware division sequence
#ifdef __CUDA_ARCH__
__device__ __noinline__ double div_other(double a, double b) { return a / b; }
#else
inline double div_other(double a, double b) { return a / b; }
#endif

// a / D.b rounded to nearest even, equal to the `/` operator
__host__ __device__ __forceinline__ double div(double a, const Divisor& D)
{
   const uint64_t A = bits(a);
   const int ea = (int)((A >> 52) & 0x7FF);
   if (!D.ok || ea == 0x7FF) return div_other(a, D.b);
   const uint64_t sign = (A & 0x8000000000000000ull) ^ D.sign;
   if ((A & 0x7FFFFFFFFFFFFFFFull) == 0) return from_bits(sign);   // +-0 / normal
   if (ea == 0) return div_other(a, D.b);                           // subnormal dividend
   const uint64_t ma = (A & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
   const uint64_t mb = D.d >> 11;
   // quotient significand in [1, 2): scale by 2^54 (ma >= mb) or 2^55
   const int s = ma < mb ? 1 : 0;
   const int e = ea - D.eb + 1023 - s;
   if (e <= 0) return div_other(a, D.b);                            // subnormal or zero quotient
   uint64_t r;
   // floor(ma * 2^(54+s) / mb) = floor(ma * 2^(65+s) / d), numerator (ma << (1+s)) * 2^64
   const uint64_t q = div_2by1(ma << (1 + s), 0, D.d, D.v, r);    // in [2^54, 2^55)
   uint64_t m = q >> 2;
   const uint64_t g = (q >> 1) & 1, low = (q & 1) | (r != 0 ? 1 : 0);
   if (g && (low || (m & 1))) m = m + 1;                            // round to nearest even
   // m in [2^52, 2^53]; 2^53 carries into the exponent (and to infinity past 2046)
   const uint64_t out = ((uint64_t)e << 52) + m - 0x10000000000000ull;
   if (e >= 0x7FF || (out >> 52) >= 0x7FF) return from_bits(sign | 0x7FF0000000000000ull);
   return from_bits(sign | out);
}

__host__ __device__ __forceinline__ double div(double a, double b) { return div(a, divisor(b)); }

// x * 2^K on the integer pipes: for a normal x whose product stays normal
// the exponent field moves by K and the significand is unchanged, which is
// exactly the rounded product; zeros stay; anything else (subnormal,
// infinite, NaN, a product that overflows or turns subnormal) goes to the
// multiply.  Equal to x * 2^K for every x.
#ifdef __CUDA_ARCH__
__device__ __noinline__ double mul_other(double x, double s) { return x * s; }
#else
inline double mul_other(double x, double s) { return x * s; }
#endif

template <int K>
__host__ __device__ __forceinline__ double scale2(double x)
{
   constexpr double kScale = K >= 0 ? double(1ull << (K >= 0 ? K : 0)) : 1.0 / double(1ull << (K < 0 ? -K : 0));
   const uint64_t u = bits(x);
   const int e = (int)((u >> 52) & 0x7FF);
   if (e >= 1 && e <= 0x7FE && e + K >= 1 && e + K <= 0x7FE) return from_bits(u + (uint64_t)((int64_t)K << 52));
   if ((u << 1) == 0) return x;   // +-0
   return mul_other(x, kScale);
}

// a * b rounded to nearest even on the integer pipes, equal to the FP64
// multiply: for normal operands with a normal product the 53-bit
// significands multiply exactly in 128 bits (each shifted to the top of a
// 64-bit word), the top 53 bits round on the next bit and the OR of the
// rest; a zero times a zero or a normal number is a signed zero; anything
// else (subnormal, infinite or NaN operands, a product that overflows or
// turns subnormal) goes to the multiply.
__host__ __device__ __forceinline__ double mul(double a, double b)
{
   constexpr uint64_t kMant = 0xFFFFFFFFFFFFFull, kHidden = 0x10000000000000ull;
   const uint64_t ua = bits(a), ub = bits(b);
   const uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
   const int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
   const bool na = (unsigned)(ea - 1) < 0x7FEu, nb = (unsigned)(eb - 1) < 0x7FEu;
   if (!na || !nb) {
      const bool za = (ua << 1) == 0, zb = (ub << 1) == 0;
      if ((za && (zb || nb)) || (zb && na)) return from_bits(sign);
      return mul_other(a, b);
   }
   int e = ea + eb - 1023;   // biased exponent of a product in [1, 2)
   const uint64_t A = ((ua & kMant) | kHidden) << 11, B = ((ub & kMant) | kHidden) << 11;
   uint64_t hi = mulhi(A, B), lo = A * B;
   if (hi >> 63) {
      e += 1;
   } else {
      hi = (hi << 1) | (lo >> 63);
      lo <<= 1;
   }
   if (e < 1) return mul_other(a, b);   // subnormal or zero product
   uint64_t m = hi >> 11;
   const uint64_t g = (hi >> 10) & 1;
   const bool st = ((hi & 0x3FF) | lo) != 0;
   if (g && (st || (m & 1))) m = m + 1;
   if (m >> 53) {
      m >>= 1;
      e += 1;
   }
   if (e > 0x7FE) return mul_other(a, b);   // overflow
   return from_bits(sign | ((uint64_t)e << 52) | (m & kMant));
}

// 0.0 + v (sub false) or 0.0 - v (sub true) on the integer pipes, equal to
// the FP64 add: +-v with the sign flipped for sub, except that a zero v
// gives +0.0 either way
__host__ __device__ __forceinline__ double zero_plus(double v, bool sub)
{
   const uint64_t u = bits(v);
   return from_bits(((u << 1) == 0) ? 0ull : (sub ? u ^ 0x8000000000000000ull : u));
}

}  // namespace sd

// a * b in the reconstructions and fluxes: with SOFT (FP64) on the integer
// pipes (sd::mul, identical results), otherwise the multiply
template <bool SOFT>
__host__ __device__ __forceinline__ double pm(double a, double b)
{
   return SOFT ? sd::mul(a, b) : a * b;
}
template <bool SOFT>
__host__ __device__ __forceinline__ float pm(float a, float b)
{
   return a * b;
}

// x * 2^K in the reconstructions: with SOFT (FP64 only) on the integer
// pipes (sd::scale2, identical results), otherwise the multiply
template <int K, bool SOFT>
__host__ __device__ __forceinline__ double p2(double x)
{
   constexpr double kScale = K >= 0 ? double(1ull << (K >= 0 ? K : 0)) : 1.0 / double(1ull << (K < 0 ? -K : 0));
   return SOFT ? sd::scale2<K>(x) : kScale * x;
}
template <int K, bool SOFT>
__host__ __device__ __forceinline__ float p2(float x)
{
   constexpr float kScale = K >= 0 ? float(1u << (K >= 0 ? K : 0)) : 1.0f / float(1u << (K < 0 ? -K : 0));
   return kScale * x;
}

// Division by one divisor, possibly several times: in FP64 with SOFT the
// correctly rounded integer-pipe division above (identical results to `/`,
// off the FP64 pipe the FP64 kernels are bound by); otherwise the
// operator.  Which is faster depends on the kernel and the mesh (the
// autotuner picks).
template <typename T, bool SOFT = true>
struct Dv {
   T b;
   __device__ __forceinline__ explicit Dv(T b_) : b(b_) {}
   __device__ __forceinline__ T div(T a) const { return a / b; }
};
template <>
struct Dv<double, true> {
   sd::Divisor D;
   __device__ __forceinline__ explicit Dv(double b) : D(sd::divisor(b)) {}
   __device__ __forceinline__ double div(double a) const { return sd::div(a, D); }
};

}  // namespace hamstr
#endif
