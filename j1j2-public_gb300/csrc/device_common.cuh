// Device building blocks of the sweep engine: Philox4x32-10, the engine's own FP64 exponential,
// the colour-compact lattice geometry and the per-site local-field arithmetic of both forms.
//
// Colour-compact layout (per lattice, in HBM and in shared memory): site (x, y, z) has colour
// c = (x&1) | (y&1)<<1 | (z&1)<<2 and compact coordinates X = x>>1, Y = y>>1, Z = z>>1; it is
// stored at ((c*Hh + Z)*Lh + Y)*Lh + X with Lh = L/2, Hh = H/2.  Every neighbour of a site
// (J:540-584: +-x, +-y, the four x-y diagonals, +-z) has another colour, so one colour class is
// updated in parallel without races, and the neighbours of a run of consecutive X of one colour
// are runs of consecutive X (shifted by at most one) of the neighbouring colours.
//
// Spins are stored biased: byte b = s + 1 (0 = down, 2 = up, 1 = vacancy, s = 0), so four
// neighbour bytes can be added inside one 32-bit word without carries.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace j1j2 {

// ------------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11).  Stream layout of the engine:
//   key = (seed, conf_base + conf)
//   sweep uniforms : ctr = (replica, sweep, group, 0), group = ((c*Hh + Z)*Lh + Y)*Qr + (X>>2),
//                    Qr = ceil(Lh/4); the site takes output word X & 3
//   swap uniforms  : ctr = (cycle, pair, 0, 1), word 0
//   HOT start      : ctr = (replica, 0, group, 2), word X & 3, s = +1 when the word < 2^31
// ------------------------------------------------------------------------------------------------
enum : uint32_t { kTagSweep = 0u, kTagSwap = 1u, kTagInit = 2u };

struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                     uint32_t c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#if defined(__CUDA_ARCH__)
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

// The same generator with its key schedule given: round r uses k0s[r] and k1s[r] + k1add, which
// equal k0 + r * 0x9E3779B9 and k1 + r * 0xBB67AE85 of philox4x32_10 for k0s[r] = k0 + r *
// 0x9E3779B9 and k1s[r] + k1add = k1 + r * 0xBB67AE85.  A kernel passes the launch-uniform part of
// the schedule among its parameters, so the rounds XOR a parameter instead of forming the key.
__device__ __forceinline__ U4 philox4x32_10_rk(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                               const uint32_t (&k0s)[10],
                                               const uint32_t (&k1s)[10], uint32_t k1add)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0s[r];
        const uint32_t n2 = hi0 ^ c3 ^ (k1s[r] + k1add);
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    return U4{c0, c1, c2, c3};
}

__host__ __device__ __forceinline__ uint32_t u4_word(const U4& v, int w)
{
    return w == 0 ? v.x : (w == 1 ? v.y : (w == 2 ? v.z : v.w));
}

// IEEE bit pattern -> double on host and device
__host__ __device__ __forceinline__ double bits_to_double(long long v)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(v);
#else
    double d;
    memcpy(&d, &v, sizeof d);
    return d;
#endif
}

// ------------------------------------------------------------------------------------------------
// FP64 exponential used by the FP64 form's acceptance tests and the PT swap.  Method: Cody-Waite
// reduction x = k*ln2 + r (ln2 split into a 32-bit head and its tail, so k*head is exact), the
// degree-13 Taylor polynomial of e^r in Horner form with fused multiply-adds, and an exact
// two-step scaling by 2^k.  Every operation is one IEEE-rounded step, so host and device give the
// same bits; the error is below one ulp over the range the sampler uses.
// ------------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ double own_exp(double x)
{
    if (x != x) return x;
    if (x > 709.8) return bits_to_double(0x7FF0000000000000ll);
    if (x < -745.2) return 0.0;
    const double inv_ln2 = 0x1.71547652b82fep+0;
    const double ln2_hi = 0x1.62e42fee00000p-1;
    const double ln2_lo = 0x1.a39ef35793c76p-33;
#if defined(__CUDA_ARCH__)
    const double kd = rint(__dmul_rn(x, inv_ln2));
    double r = __fma_rn(-kd, ln2_hi, x);
    r = __fma_rn(-kd, ln2_lo, r);
#define J1J2_FMA __fma_rn
#else
    const double kd = nearbyint(x * inv_ln2);
    double r = fma(-kd, ln2_hi, x);
    r = fma(-kd, ln2_lo, r);
#define J1J2_FMA fma
#endif
    double q = 0x1.6124613a86d09p-33;  // 1/13!
    q = J1J2_FMA(q, r, 0x1.1eed8eff8d898p-29);
    q = J1J2_FMA(q, r, 0x1.ae64567f544e4p-26);
    q = J1J2_FMA(q, r, 0x1.27e4fb7789f5cp-22);
    q = J1J2_FMA(q, r, 0x1.71de3a556c734p-19);
    q = J1J2_FMA(q, r, 0x1.a01a01a01a01ap-16);
    q = J1J2_FMA(q, r, 0x1.a01a01a01a01ap-13);
    q = J1J2_FMA(q, r, 0x1.6c16c16c16c17p-10);
    q = J1J2_FMA(q, r, 0x1.1111111111111p-7);
    q = J1J2_FMA(q, r, 0x1.5555555555555p-5);
    q = J1J2_FMA(q, r, 0x1.5555555555555p-3);
    q = J1J2_FMA(q, r, 0.5);
    q = J1J2_FMA(q, r, 1.0);
    q = J1J2_FMA(q, r, 1.0);
#undef J1J2_FMA
    const int k = (int)kd;
    const int k1 = k / 2, k2 = k - k1;
    const double s1 = bits_to_double((long long)(k1 + 1023) << 52);
    const double s2 = bits_to_double((long long)(k2 + 1023) << 52);
#if defined(__CUDA_ARCH__)
    return __dmul_rn(__dmul_rn(q, s1), s2);
#else
    return (q * s1) * s2;
#endif
}

// ------------------------------------------------------------------------------------------------
// Geometry of one lattice shape
// ------------------------------------------------------------------------------------------------
struct Geo {
    int L, H;    // lattice extents
    int Lh, Hh;  // L/2, H/2
    int N;       // sites
    int Nc;      // sites per colour (Lh*Lh*Hh)
    int Qr;      // Philox groups per compact row, ceil(Lh/4)
};

__host__ __device__ __forceinline__ int cidx(const Geo& g, int c, int Z, int Y, int X)
{
    return ((c * g.Hh + Z) * g.Lh + Y) * g.Lh + X;
}

// Canonical site (x + L*y + L*L*z) -> compact index
__host__ __device__ __forceinline__ int compact_of_site(const Geo& g, int site)
{
    const int x = site % g.L, y = (site / g.L) % g.L, z = site / (g.L * g.L);
    const int c = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
    return cidx(g, c, z >> 1, y >> 1, x >> 1);
}

// ------------------------------------------------------------------------------------------------
// FP64 local field in the operation order of Compute_local_field (J:2498-2541).  Spins s1..s10
// are the neighbours m1..m10 (+y, -y, +x, -x, (+x,+y), (-x,+y), (+x,-y), (-x,-y), +z, -z) as
// -1/0/+1; a vacancy neighbour (s = 0) contributes signed zeros, which leaves every partial sum
// bit-identical to skipping it as the reference's occu() gates do (no partial sum is -0).
// Products of a spin with a coupling are exact; only the additions round, in the same order.
// ------------------------------------------------------------------------------------------------
struct Nbr64 {
    int s[10];
    double p1, p2, p3, p4;  // p at m1..m4
    int jv_own, jv_m2, jh_own, jh_m4;
};

// s * c for a spin s in {-1, 0, +1}: the product is exact, so it is a selection of c's bits with
// the sign flipped for s = -1, in integer operations rather than on the FP64 pipe (GB300 runs 2
// FP64 operations per clock per SM; a negation there would cost as much as the addition).  A
// vacancy's zero is +0; since no partial sum is -0, adding it leaves the sum as IEEE
// multiplication's signed zero would.
__device__ __forceinline__ double spin_mul(int s, double c)
{
    const int hi = __double2hiint(c) ^ (s < 0 ? (int)0x80000000 : 0);
    return __hiloint2double(s == 0 ? 0 : hi, s == 0 ? 0 : __double2loint(c));
}

// A small integer n (|n| <= 15) as a double, built from its bits (no FP64 conversion)
__device__ __forceinline__ double small_int_double(int n)
{
    const int m = n < 0 ? -n : n;
    if (m == 0) return 0.0;
    const int e = 31 - __clz(m);  // m = 2^e (1 + f)
    const int hi = ((1023 + e) << 20) | ((m << (20 - e)) & 0xFFFFF);
    return __hiloint2double(n < 0 ? hi | (int)0x80000000 : hi, 0);
}

// s f <= 0 for a spin s = +-1: the Metropolis move is downhill (or level) and accepted without a
// random number; read off the sign bit of f (and f = +-0) without an FP64 comparison
__device__ __forceinline__ bool downhill(double f, int s)
{
    const long long b = __double_as_longlong(f);
    return (b << 1) == 0 || ((b < 0) == (s == 1));
}

__device__ __forceinline__ double field_fp64(const Nbr64& n, double pi, double J1h, double J1v,
                                             double J2, double J3, double* nem_out)
{
    // 0 + t = t exactly (up to the sign of a zero, which no later sum or test can see)
    double f = n.jv_own ? spin_mul(n.s[0], J1v) : 0.0;
    f = __dsub_rn(f, spin_mul(n.s[0], n.p1));
    f = __dadd_rn(f, n.jv_m2 ? spin_mul(n.s[1], J1v) : 0.0);
    f = __dsub_rn(f, spin_mul(n.s[1], n.p2));
    f = __dadd_rn(f, n.jh_own ? spin_mul(n.s[2], J1h) : 0.0);
    f = __dadd_rn(f, spin_mul(n.s[2], n.p3));
    f = __dadd_rn(f, n.jh_m4 ? spin_mul(n.s[3], J1h) : 0.0);
    f = __dadd_rn(f, spin_mul(n.s[3], n.p4));
#pragma unroll
    for (int k = 4; k < 8; ++k) f = __dadd_rn(f, spin_mul(n.s[k], J2));
#pragma unroll
    for (int k = 8; k < 10; ++k) f = __dadd_rn(f, spin_mul(n.s[k], J3));
    // the nematic sum -s1 - s2 + s3 + s4 is an exact small integer in any order
    const double nm = small_int_double(n.s[2] + n.s[3] - n.s[0] - n.s[1]);
    f = __dadd_rn(f, __dmul_rn(pi, nm));
    if (nem_out) *nem_out = nm;
    return f;
}

// ------------------------------------------------------------------------------------------------
// FP32 local field (the batched form).  Same Hamiltonian written per bond:
//   field = sum_x (J1h*jh + p_i + p_j) s_j + sum_y (J1v*jv - p_i - p_j) s_j + J2*D + J3*Zs
// with D the sum of the four diagonal spins and Zs the sum of the two inter-layer spins.
// ------------------------------------------------------------------------------------------------
struct Nbr32 {
    float sxp, sxm, syp, sym;  // spins at +x, -x, +y, -y
    float D, Zs;               // diagonal and inter-layer spin sums
    float pxp, pxm, pyp, pym;  // p at +x, -x, +y, -y
};

__device__ __forceinline__ float field_fp32(const Nbr32& n, float pi, float J1h, float J1v,
                                            float J2, float J3)
{
    const float sx = n.sxp + n.sxm, sy = n.syp + n.sym;
    float f = __fmul_rn(J3, n.Zs);
    f = __fmaf_rn(J2, n.D, f);
    f = __fmaf_rn(__fadd_rn(J1h, pi), sx, f);
    f = __fmaf_rn(__fsub_rn(J1v, pi), sy, f);
    f = __fmaf_rn(n.pxp, n.sxp, f);
    f = __fmaf_rn(n.pxm, n.sxm, f);
    f = __fmaf_rn(-n.pyp, n.syp, f);
    f = __fmaf_rn(-n.pym, n.sym, f);
    return f;
}

// Same with diluted bonds: jh_own/jh_m4 gate the J1h terms of the +x / -x bonds, jv_own/jv_m2
// the J1v terms of the +y / -y bonds (J:2511-2532); the phi terms are not gated.
__device__ __forceinline__ float field_fp32_masked(const Nbr32& n, float pi, float J1h, float J1v,
                                                   float J2, float J3, float jh_own, float jh_m4,
                                                   float jv_own, float jv_m2)
{
    const float sx = n.sxp + n.sxm, sy = n.syp + n.sym;
    const float hx = __fmaf_rn(jh_own, n.sxp, __fmul_rn(jh_m4, n.sxm));
    const float hy = __fmaf_rn(jv_own, n.syp, __fmul_rn(jv_m2, n.sym));
    float f = __fmul_rn(J3, n.Zs);
    f = __fmaf_rn(J2, n.D, f);
    f = __fmaf_rn(J1h, hx, f);
    f = __fmaf_rn(J1v, hy, f);
    f = __fmaf_rn(pi, __fsub_rn(sx, sy), f);
    f = __fmaf_rn(n.pxp, n.sxp, f);
    f = __fmaf_rn(n.pxm, n.sxm, f);
    f = __fmaf_rn(-n.pyp, n.syp, f);
    f = __fmaf_rn(-n.pym, n.sym, f);
    return f;
}

// 2^x with the SFU (ex2.approx.ftz.f32)
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// FP64 uniform in [0, 1) from a Philox word: the word rotated left by 9 bits, times 2^-32.  Its
// top 23 bits are the word's low 23 bits, i.e. exactly the FP32 uniform below, so both forms
// test the same random number (to 2^-23) in the deterministic FP32-vs-FP64 replay.
__host__ __device__ __forceinline__ double u01_f64(uint32_t r)
{
    return (double)((r << 9) | (r >> 23)) * 0x1p-32;
}

// FP64 Metropolis test u < own_exp(x) for u = u01_f64(r) and x < 0, decided from an FP32
// estimate of exp(x) unless u lies inside the estimate's error band, where own_exp decides: the
// result is exactly that of u01_f64(r) < own_exp(x).  Error of the estimate 2^(x log2e) for
// -80 <= x <= 0 (no FP32 underflow; the cut is taken on x rounded to FP32, which moves it by
// 2^-18 at most): rounding x and the product to FP32 shifts the exponent by at most
// |x| (2^-24 + 2^-23), and the SFU's ex2 is taken at 2^-20 relative (above its documented
// accuracy); the band e (|x| 2^-20 + 2^-18) is four times the sum.  The comparisons with the
// band's ends need no FP64 arithmetic (GB300 runs 2 FP64 operations per clock per SM): u is the
// integer v = rotl(r, 9) times 2^-32, and for a float y >= 0 (y 2^32 exact in FP32)
// u < y  <=>  v < ceil(y 2^32)  and  u > y  <=>  v > floor(y 2^32); the conversions saturate
// at 2^32 - 1, where the first test is settled by y >= 1 beforehand and the second is false, as
// u > y is for y >= 1.
__device__ __forceinline__ bool accept_fp64(uint32_t r, double x)
{
    const float xf = __double2float_rn(x);
    if (xf >= -80.0f) {
        const uint32_t v = (r << 9) | (r >> 23);
        const float e = ex2_approx(__fmul_rn(xf, 1.44269504f));
        const float band = __fmul_rn(e, __fmaf_rn(fabsf(xf), 0x1p-20f, 0x1p-18f));
        const float lo = __fsub_rn(e, band), hi = __fadd_rn(e, band);
        if (lo >= 1.0f || v < __float2uint_ru(__fmul_rn(lo, 0x1p32f))) return true;
        if (v > __float2uint_rd(__fmul_rn(hi, 0x1p32f))) return false;
    }
    return u01_f64(r) < own_exp(x);
}

// x = -2 f beta * s for the spin s = +-1 of a site whose field f is nonzero (and, as a sum of
// couplings of order one, normal): the doubling is exact, so it is an exponent increment
__device__ __forceinline__ double metropolis_arg(double f, double beta, int s)
{
    const double f2 = __hiloint2double(__double2hiint(f) + 0x00100000, __double2loint(f));
    return spin_mul(-s, __dmul_rn(f2, beta));
}

// FP32 uniform in [0, 1) from a Philox word: its low 23 bits as a mantissa, (r mod 2^23) * 2^-23
// (one logic operation; every Philox output bit is equally random)
__device__ __forceinline__ float u01_f32(uint32_t r)
{
    return __fsub_rn(__uint_as_float(0x3F800000u | (r & 0x007FFFFFu)), 1.0f);
}

// byte k of w as an exact float (b in 0..255)
__device__ __forceinline__ float byte_f(uint32_t w, int k)
{
    return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + (uint32_t)k)),
                     8388608.0f);
}

}  // namespace j1j2
