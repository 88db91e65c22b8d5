// sm_103a kernels of the engine:
//   sweep_kernel  one CTA per lattice: stage the lattice in shared memory, run the fused sweeps
//                 of one PT cycle colour by colour (8 colour phases per sweep, one barrier each),
//                 reduce the observables of the new configuration, write the lattice back.
//                 Replaces Metro_sweep / Compute_local_field (J:2498-2608) and Measurement /
//                 Spatial_mean_local_nematic (J:2807-2842, J:1028-1048).
//   swap_kernel   one CTA for all confs: observables, the odd/even adjacent replica exchange of
//                 Pt_attempt_swaps (J:1303-1338), visit flags and the per-slot running sums of
//                 Pt_measurement_loop (J:1440-1513).
//   init_kernel   HOT/FER/STR starts (Initialize_spin_array J:1179-1209) on the device.
#include <cooperative_groups.h>

#include "sweep_common.cuh"

namespace cg = cooperative_groups;

namespace j1j2 {
namespace {

// ------------------------------------------------------------------------------------------------
// Per-site path (any even L, H): one site per thread per colour phase.
// ------------------------------------------------------------------------------------------------
// Spin bytes of a lattice held whole in one array of the compact layout (shared or global
// memory); site_step reads and writes spins through such an accessor (the cluster path's reaches
// into the neighbouring CTAs' shared memory).
struct FlatBytes {
    uint8_t* S;
    __device__ __forceinline__ int get(int i, int, int, int, int) const { return S[i]; }
    __device__ __forceinline__ void set(int i, int, int, int, int, uint8_t v) const { S[i] = v; }
};

template <class Real, bool MASKS, int MODE, bool MEASURE, class Bytes>
__device__ __forceinline__ void site_step(const SweepArgs& a, const Geo& g, const Bytes& S,
                                          const Real* P, const uint8_t* BM, const float* Pf32,
                                          int c, int X, int Y, int Z, uint32_t sweep, uint32_t rep,
                                          uint32_t k0, uint32_t k1, double beta, float kb,
                                          Acc& acc, int* fl = nullptr)
{
    const int px = c & 1, py = (c >> 1) & 1, pz = c >> 2;
    const int Xp = px ? wrap_p(X, g.Lh) : X, Xm = px ? X : wrap_m(X, g.Lh);
    const int Yp = py ? wrap_p(Y, g.Lh) : Y, Ym = py ? Y : wrap_m(Y, g.Lh);
    const int Zp = pz ? wrap_p(Z, g.Hh) : Z, Zm = pz ? Z : wrap_m(Z, g.Hh);
    const int i = cidx(g, c, Z, Y, X);
    const int b = S.get(i, c, Z, Y, X);
    if (b == 1) return;  // vacancy: no attempt and no measured term (J:2563, J:2825)
    const int i1 = cidx(g, c ^ 2, Z, Yp, X), i2 = cidx(g, c ^ 2, Z, Ym, X);
    const int i3 = cidx(g, c ^ 1, Z, Y, Xp), i4 = cidx(g, c ^ 1, Z, Y, Xm);
    const int i5 = cidx(g, c ^ 3, Z, Yp, Xp), i6 = cidx(g, c ^ 3, Z, Yp, Xm);
    const int i7 = cidx(g, c ^ 3, Z, Ym, Xp), i8 = cidx(g, c ^ 3, Z, Ym, Xm);
    const int i9 = cidx(g, c ^ 4, Zp, Y, X), i10 = cidx(g, c ^ 4, Zm, Y, X);
    const int b1 = S.get(i1, c ^ 2, Z, Yp, X), b2 = S.get(i2, c ^ 2, Z, Ym, X);
    const int b3 = S.get(i3, c ^ 1, Z, Y, Xp), b4 = S.get(i4, c ^ 1, Z, Y, Xm);
    const int b5 = S.get(i5, c ^ 3, Z, Yp, Xp), b6 = S.get(i6, c ^ 3, Z, Yp, Xm);
    const int b7 = S.get(i7, c ^ 3, Z, Ym, Xp), b8 = S.get(i8, c ^ 3, Z, Ym, Xm);
    const int b9 = S.get(i9, c ^ 4, Zp, Y, X), b10 = S.get(i10, c ^ 4, Zm, Y, X);
    const int s = b - 1;
    int jh_own = 1, jh_m4 = 1, jv_own = 1, jv_m2 = 1;
    if constexpr (MASKS) {
        jh_own = BM[i] & 1;
        jv_own = (BM[i] >> 1) & 1;
        jh_m4 = BM[i4] & 1;
        jv_m2 = (BM[i2] >> 1) & 1;
    }

    if constexpr (MEASURE) {
        acc.M += s;
        acc.SX += px ? -s : s;
        acc.SY += py ? -s : s;
        acc.NB += s * (b3 + b4 - b1 - b2);
    }

    bool flip64 = false;
    double f64 = 0.0;
    if constexpr (sizeof(Real) == 8) {
        Nbr64 n;
        n.s[0] = b1 - 1;
        n.s[1] = b2 - 1;
        n.s[2] = b3 - 1;
        n.s[3] = b4 - 1;
        n.s[4] = b5 - 1;
        n.s[5] = b6 - 1;
        n.s[6] = b7 - 1;
        n.s[7] = b8 - 1;
        n.s[8] = b9 - 1;
        n.s[9] = b10 - 1;
        n.p1 = P[i1];
        n.p2 = P[i2];
        n.p3 = P[i3];
        n.p4 = P[i4];
        n.jv_own = jv_own;
        n.jv_m2 = jv_m2;
        n.jh_own = jh_own;
        n.jh_m4 = jh_m4;
        f64 = field_fp64(n, P[i], a.J1h, a.J1v, a.J2, a.J3, nullptr);
        if constexpr (MEASURE) {
            acc.e += efix(spin_mul(-s, f64));
            return;
        }
    }

    // FP32 field (the FP32 form, or the FP32 side of the audit)
    float f32 = 0.0f;
    if constexpr (sizeof(Real) == 4 || MODE == kModeAudit) {
        const float* Q;
        if constexpr (sizeof(Real) == 4)
            Q = reinterpret_cast<const float*>(P);
        else
            Q = Pf32;
        Nbr32 n;
        n.syp = (float)(b1 - 1);
        n.sym = (float)(b2 - 1);
        n.sxp = (float)(b3 - 1);
        n.sxm = (float)(b4 - 1);
        n.D = (float)(b5 + b6 + b7 + b8 - 4);
        n.Zs = (float)(b9 + b10 - 2);
        n.pyp = Q[i1];
        n.pym = Q[i2];
        n.pxp = Q[i3];
        n.pxm = Q[i4];
        if constexpr (MASKS)
            f32 = field_fp32_masked(n, Q[i], a.J1hf, a.J1vf, a.J2f, a.J3f, (float)jh_own,
                                    (float)jh_m4, (float)jv_own, (float)jv_m2);
        else
            f32 = field_fp32(n, Q[i], a.J1hf, a.J1vf, a.J2f, a.J3f);
        if constexpr (MEASURE && sizeof(Real) == 4) {
            acc.e += efix32(-__fmul_rn((float)s, f32));
            return;
        }
    }

    const uint32_t grp = (uint32_t)(((c * g.Hh + Z) * g.Lh + Y) * g.Qr + (X >> 2));
    const int w = X & 3;
    uint32_t r = 0;
    if constexpr (sizeof(Real) == 8) {
        // FP64 acceptance, J:2572-2604: no uniform is needed when dE <= 0
        if (downhill(f64, s)) {
            flip64 = true;
        } else {
            r = u4_word(philox4x32_10(rep, sweep, grp, kTagSweep, k0, k1), w);
            flip64 = accept_fp64(r, metropolis_arg(f64, beta, s));
        }
        if constexpr (MODE == kModeAudit) {
            r = u4_word(philox4x32_10(rep, sweep, grp, kTagSweep, k0, k1), w);
            const float sf = __fmul_rn((float)s, f32);
            const bool flip32 = u01_f32(r) < ex2_approx(__fmul_rn(kb, sf));
            acc.M += 1;
            acc.SX += (flip32 != flip64);
        }
        if (flip64) {
            S.set(i, c, Z, Y, X, (uint8_t)(2 - b));
            if (fl) fl[i] += 1;
        }
    } else {
        r = u4_word(philox4x32_10(rep, sweep, grp, kTagSweep, k0, k1), w);
        const float sf = __fmul_rn((float)s, f32);
        if (u01_f32(r) < ex2_approx(__fmul_rn(kb, sf))) {
            S.set(i, c, Z, Y, X, (uint8_t)(2 - b));
            if (fl) fl[i] += 1;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Quad path (Lh % 4 == 0): a thread owns four consecutive compact X of one colour in one row,
// i.e. one 32-bit word of spins and one Philox call (four uniforms).  Its neighbours are whole
// words of the neighbouring colours, or words shifted by one byte (__byte_perm with the next /
// previous word); diagonal and inter-layer neighbours are summed bytewise in 32-bit adds.
// ------------------------------------------------------------------------------------------------
struct QuadNbr {
    uint32_t own, xp, xm, yp, ym, dpp, dpm, dmp, dmm, zp, zm;
};

// Flip-count row of the replica's temperature slot (nullptr: flips are not counted)
__device__ __forceinline__ int* flip_row(const SweepArgs& a, int conf, int rep)
{
    if (!a.flips || a.use_override) return nullptr;
    return a.flips + ((long long)conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]) * a.lat_stride;
}

// Spin words of a lattice held whole in one array of the compact layout (shared or global memory)
struct CompactSpins {
    uint32_t* S32;
    int rowstride, colstride, Qr;  // words per compact z-plane, per colour, per row
    __device__ __forceinline__ CompactSpins(uint32_t* s, const Geo& g)
        : S32(s), rowstride(g.Lh * g.Qr), colstride(g.Hh * g.Lh * g.Qr), Qr(g.Qr)
    {
    }
    __device__ __forceinline__ uint32_t word(int cc, int ZZ, int YY, int qq) const
    {
        return S32[cc * colstride + ZZ * rowstride + YY * Qr + qq];
    }
    __device__ __forceinline__ void put(int cc, int ZZ, int YY, int qq, uint32_t v) const
    {
        S32[cc * colstride + ZZ * rowstride + YY * Qr + qq] = v;
    }
};

template <class Real, bool MASKS, bool MEASURE, class Spins>
__device__ __forceinline__ void quad_step(const SweepArgs& a, const Geo& g, const Spins& sp,
                                          const Real* P, const uint8_t* BM, int c, int q,
                                          uint32_t sweep, uint32_t rep, uint32_t k0, uint32_t k1,
                                          double beta, float kb, Acc& acc, int* fl = nullptr)
{
    const int Qr = g.Qr;
    const int row = q / Qr;
    const int qx = q - row * Qr;
    const int Z = row / g.Lh;
    const int Y = row - Z * g.Lh;
    const int px = c & 1, py = (c >> 1) & 1, pz = c >> 2;
    const int Yp = py ? wrap_p(Y, g.Lh) : Y, Ym = py ? Y : wrap_m(Y, g.Lh);
    const int Zp = pz ? wrap_p(Z, g.Hh) : Z, Zm = pz ? Z : wrap_m(Z, g.Hh);
    const int qn = px ? wrap_p(qx, Qr) : wrap_m(qx, Qr);
    const int rowstride = g.Lh * Qr;       // words per compact z-plane
    const int colstride = g.Hh * rowstride;  // words per colour
    auto W = [&](int cc, int ZZ, int YY, int qq) {
        return cc * colstride + ZZ * rowstride + YY * Qr + qq;
    };
    QuadNbr n;
    const int wown = W(c, Z, Y, qx);
    n.own = sp.word(c, Z, Y, qx);
    x_pair(px, sp.word(c ^ 1, Z, Y, qx), sp.word(c ^ 1, Z, Y, qn), n.xp, n.xm);
    n.yp = sp.word(c ^ 2, Z, Yp, qx);
    n.ym = sp.word(c ^ 2, Z, Ym, qx);
    x_pair(px, sp.word(c ^ 3, Z, Yp, qx), sp.word(c ^ 3, Z, Yp, qn), n.dpp, n.dpm);
    x_pair(px, sp.word(c ^ 3, Z, Ym, qx), sp.word(c ^ 3, Z, Ym, qn), n.dmp, n.dmm);
    n.zp = sp.word(c ^ 4, Zp, Y, qx);
    n.zm = sp.word(c ^ 4, Zm, Y, qx);

    uint32_t mown = 0xFFFFFFFFu, mxm = 0xFFFFFFFFu, mym = 0xFFFFFFFFu;
    if constexpr (MASKS) {
        const uint32_t* BM32 = reinterpret_cast<const uint32_t*>(BM);
        mown = BM32[wown];
        uint32_t dummy;
        x_pair(px, BM32[W(c ^ 1, Z, Y, qx)], BM32[W(c ^ 1, Z, Y, qn)], dummy, mxm);
        mym = BM32[W(c ^ 2, Z, Ym, qx)];
    }

    // random field: own, x neighbours (same word and one shifted element), y rows
    Real pown[4], pxa[4], pyp[4], pym[4];
    const int X0 = 4 * qx;
    const int bo = cidx(g, c, Z, Y, X0), bx = cidx(g, c ^ 1, Z, Y, X0);
    const int byp = cidx(g, c ^ 2, Z, Yp, X0), bym = cidx(g, c ^ 2, Z, Ym, X0);
    const Real pextra = P[cidx(g, c ^ 1, Z, Y, px ? 4 * qn : 4 * qn + 3)];
    if constexpr (sizeof(Real) == 4) {
        const float4 v0 = *reinterpret_cast<const float4*>(P + bo);
        const float4 v1 = *reinterpret_cast<const float4*>(P + bx);
        const float4 v2 = *reinterpret_cast<const float4*>(P + byp);
        const float4 v3 = *reinterpret_cast<const float4*>(P + bym);
        pown[0] = v0.x, pown[1] = v0.y, pown[2] = v0.z, pown[3] = v0.w;
        pxa[0] = v1.x, pxa[1] = v1.y, pxa[2] = v1.z, pxa[3] = v1.w;
        pyp[0] = v2.x, pyp[1] = v2.y, pyp[2] = v2.z, pyp[3] = v2.w;
        pym[0] = v3.x, pym[1] = v3.y, pym[2] = v3.z, pym[3] = v3.w;
    } else {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const double2 v0 = *reinterpret_cast<const double2*>(P + bo + 2 * h);
            const double2 v1 = *reinterpret_cast<const double2*>(P + bx + 2 * h);
            const double2 v2 = *reinterpret_cast<const double2*>(P + byp + 2 * h);
            const double2 v3 = *reinterpret_cast<const double2*>(P + bym + 2 * h);
            pown[2 * h] = v0.x, pown[2 * h + 1] = v0.y;
            pxa[2 * h] = v1.x, pxa[2 * h + 1] = v1.y;
            pyp[2 * h] = v2.x, pyp[2 * h + 1] = v2.y;
            pym[2 * h] = v3.x, pym[2 * h + 1] = v3.y;
        }
    }

    U4 rnd{0, 0, 0, 0};
    if constexpr (!MEASURE) {
        const uint32_t grp = (uint32_t)(c * colstride + q);
        rnd = philox4x32_10(rep, sweep, grp, kTagSweep, k0, k1);
    }
    uint32_t flipmask = 0;
    const uint32_t dsum = n.dpp + n.dpm + n.dmp + n.dmm;  // bytewise, <= 8 each
    const uint32_t zsum = n.zp + n.zm;                    // bytewise, <= 4 each
    if constexpr (sizeof(Real) == 4 && !MEASURE) {
        // Sweep in pairs of sites with packed FP32x2 arithmetic, element by element the
        // operations and rounding of field_fp32 / field_fp32_masked (-y terms as products with
        // the negated spins, exactly).
        const f2 c1 = f2_splat(8388609.0f), c2 = f2_splat(8388610.0f), c4 = f2_splat(8388612.0f);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * h;
            const f2 sxp = f2_sub(byte_pair(n.xp, k), c1);
            const f2 sxm = f2_sub(byte_pair(n.xm, k), c1);
            const f2 nsyp = f2_sub(c1, byte_pair(n.yp, k));
            const f2 nsym = f2_sub(c1, byte_pair(n.ym, k));
            const f2 D = f2_sub(byte_pair(dsum, k), c4);
            const f2 Zs = f2_sub(byte_pair(zsum, k), c2);
            const f2 si = f2_sub(byte_pair(n.own, k), c1);
            const f2 pi = f2_pack(pown[k], pown[k + 1]);
            const f2 pxp = px ? f2_pack(pxa[k + 1], k + 1 < 3 ? pxa[k + 2] : pextra)
                              : f2_pack(pxa[k], pxa[k + 1]);
            const f2 pxm = px ? f2_pack(pxa[k], pxa[k + 1])
                              : f2_pack(k > 0 ? pxa[k - 1] : pextra, pxa[k]);
            const f2 pyp2 = f2_pack(pyp[k], pyp[k + 1]);
            const f2 pym2 = f2_pack(pym[k], pym[k + 1]);
            const f2 sx = f2_add(sxp, sxm), nsy = f2_add(nsyp, nsym);
            f2 f = f2_mul(f2_splat(a.J3f), Zs);
            f = f2_fma(f2_splat(a.J2f), D, f);
            if constexpr (MASKS) {
                const int sh0 = 8 * k, sh1 = 8 * k + 8;
                const f2 jho = f2_pack((float)((mown >> sh0) & 1), (float)((mown >> sh1) & 1));
                const f2 jhm = f2_pack((float)((mxm >> sh0) & 1), (float)((mxm >> sh1) & 1));
                const f2 jvo = f2_pack((float)((mown >> (sh0 + 1)) & 1),
                                       (float)((mown >> (sh1 + 1)) & 1));
                const f2 jvm = f2_pack((float)((mym >> (sh0 + 1)) & 1),
                                       (float)((mym >> (sh1 + 1)) & 1));
                const f2 hx = f2_fma(jho, sxp, f2_mul(jhm, sxm));
                const f2 nhy = f2_fma(jvo, nsyp, f2_mul(jvm, nsym));  // -hy
                f = f2_fma(f2_splat(a.J1hf), hx, f);
                f = f2_fma(f2_splat(-a.J1vf), nhy, f);
                f = f2_fma(pi, f2_add(sx, nsy), f);
            } else {
                f = f2_fma(f2_add(f2_splat(a.J1hf), pi), sx, f);
                f = f2_fma(f2_sub(pi, f2_splat(a.J1vf)), nsy, f);
            }
            f = f2_fma(pxp, sxp, f);
            f = f2_fma(pxm, sxm, f);
            f = f2_fma(pyp2, nsyp, f);
            f = f2_fma(pym2, nsym, f);
            const f2 sf = f2_mul(si, f);
            const f2 arg = f2_mul(f2_splat(kb), sf);
            // vacancies (s = 0) never flip: the threshold is scaled by s^2
            const f2 thr = f2_mul(f2_pack(ex2_approx(f2_get(arg, 0)), ex2_approx(f2_get(arg, 1))),
                                  f2_mul(si, si));
            const f2 u = f2_sub(
                f2_pack(__uint_as_float(0x3F800000u | (u4_word(rnd, k) & 0x007FFFFFu)),
                        __uint_as_float(0x3F800000u | (u4_word(rnd, k + 1) & 0x007FFFFFu))),
                f2_splat(1.0f));
            if (f2_get(u, 0) < f2_get(thr, 0)) flipmask |= 2u << (8 * k);
            if (f2_get(u, 1) < f2_get(thr, 1)) flipmask |= 2u << (8 * k + 8);
        }
        if (flipmask) {
            sp.put(c, Z, Y, qx, n.own ^ flipmask);
            if (fl) {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if ((flipmask >> (8 * k + 1)) & 1u) fl[bo + k] += 1;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int sh = 8 * k;
            const int b = (n.own >> sh) & 0xFF;
            const Real pxp = px ? (k < 3 ? pxa[k + 1] : pextra) : pxa[k];
            const Real pxm = px ? pxa[k] : (k > 0 ? pxa[k - 1] : pextra);
            const int jh_own = (mown >> sh) & 1, jv_own = (mown >> (sh + 1)) & 1;
            const int jh_m4 = (mxm >> sh) & 1, jv_m2 = (mym >> (sh + 1)) & 1;
            if constexpr (sizeof(Real) == 4) {
                Nbr32 nb;
                nb.sxp = byte_f(n.xp, k) - 1.0f;
                nb.sxm = byte_f(n.xm, k) - 1.0f;
                nb.syp = byte_f(n.yp, k) - 1.0f;
                nb.sym = byte_f(n.ym, k) - 1.0f;
                nb.D = byte_f(dsum, k) - 4.0f;
                nb.Zs = byte_f(zsum, k) - 2.0f;
                nb.pxp = pxp;
                nb.pxm = pxm;
                nb.pyp = pyp[k];
                nb.pym = pym[k];
                float f;
                if constexpr (MASKS)
                    f = field_fp32_masked(nb, pown[k], a.J1hf, a.J1vf, a.J2f, a.J3f, (float)jh_own,
                                          (float)jh_m4, (float)jv_own, (float)jv_m2);
                else
                    f = field_fp32(nb, pown[k], a.J1hf, a.J1vf, a.J2f, a.J3f);
                const float sf = __fmul_rn((float)(b - 1), f);
                if constexpr (MEASURE) {
                    const int s = b - 1;
                    acc.e += efix32(-sf);
                    acc.M += s;
                    acc.SX += px ? -s : s;
                    acc.SY += py ? -s : s;
                    acc.NB += s * ((int)((n.xp >> sh) & 0xFF) + (int)((n.xm >> sh) & 0xFF) -
                                   (int)((n.yp >> sh) & 0xFF) - (int)((n.ym >> sh) & 0xFF));
                } else {
                    // vacancies (s = 0) never flip: the threshold is scaled by s^2
                    const float s2 = byte_f(n.own, k) - 1.0f;
                    const bool flip = u01_f32(u4_word(rnd, k)) <
                                      __fmul_rn(ex2_approx(__fmul_rn(kb, sf)), __fmul_rn(s2, s2));
                    flipmask |= flip ? (2u << sh) : 0u;
                }
            } else {
                if (b == 1) continue;
                Nbr64 nb;
                nb.s[0] = (int)((n.yp >> sh) & 0xFF) - 1;
                nb.s[1] = (int)((n.ym >> sh) & 0xFF) - 1;
                nb.s[2] = (int)((n.xp >> sh) & 0xFF) - 1;
                nb.s[3] = (int)((n.xm >> sh) & 0xFF) - 1;
                nb.s[4] = (int)((n.dpp >> sh) & 0xFF) - 1;
                nb.s[5] = (int)((n.dpm >> sh) & 0xFF) - 1;
                nb.s[6] = (int)((n.dmp >> sh) & 0xFF) - 1;
                nb.s[7] = (int)((n.dmm >> sh) & 0xFF) - 1;
                nb.s[8] = (int)((n.zp >> sh) & 0xFF) - 1;
                nb.s[9] = (int)((n.zm >> sh) & 0xFF) - 1;
                nb.p1 = pyp[k];
                nb.p2 = pym[k];
                nb.p3 = pxp;
                nb.p4 = pxm;
                nb.jv_own = jv_own;
                nb.jv_m2 = jv_m2;
                nb.jh_own = jh_own;
                nb.jh_m4 = jh_m4;
                const double f = field_fp64(nb, pown[k], a.J1h, a.J1v, a.J2, a.J3, nullptr);
                const int s = b - 1;
                if constexpr (MEASURE) {
                    acc.e += efix(spin_mul(-s, f));
                    acc.M += s;
                    acc.SX += px ? -s : s;
                    acc.SY += py ? -s : s;
                    acc.NB += s * (nb.s[2] + nb.s[3] - nb.s[0] - nb.s[1]);
                } else {
                    bool flip;
                    if (downhill(f, s)) {
                        flip = true;
                    } else {
                        flip = accept_fp64(u4_word(rnd, k), metropolis_arg(f, beta, s));
                    }
                    flipmask |= flip ? (2u << sh) : 0u;
                }
            }
        }
        if constexpr (!MEASURE) {
            if (flipmask) {
                sp.put(c, Z, Y, qx, n.own ^ flipmask);
                if (fl) {
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if ((flipmask >> (8 * k + 1)) & 1u) fl[bo + k] += 1;
                }
            }
        }
    }
}

template <class Real, bool QUAD, bool STAGE_P, bool MASKS, int MODE>
__global__ void __launch_bounds__(1024) sweep_kernel(SweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const Geo g = a.g;
    const int lat = a.lat0 + (int)blockIdx.x;
    const int conf = lat / a.nrep;
    const int rep = lat - conf * a.nrep;
    const int tid = (int)threadIdx.x, NT = (int)blockDim.x;
    const int Nb = (g.N + 15) & ~15;
    uint8_t* S = smem;
    Real* Ps = reinterpret_cast<Real*>(smem + Nb);
    uint8_t* Sg = a.spins + (long long)lat * a.lat_stride;
    const Real* Pg = field_base<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    const float* Pf32 = (MODE == kModeAudit) ? a.pf + (long long)conf * a.p_stride : nullptr;

    {  // stage the lattice (and the random field) in shared memory with 16-byte vectors
        const uint4* src = reinterpret_cast<const uint4*>(Sg);
        uint4* dst = reinterpret_cast<uint4*>(S);
        for (int k = tid; k < Nb / 16; k += NT) dst[k] = src[k];
        if constexpr (STAGE_P) {
            const int nv = (int)((g.N * sizeof(Real) + 15) / 16);
            const uint4* ps = reinterpret_cast<const uint4*>(Pg);
            uint4* pdst = reinterpret_cast<uint4*>(Ps);
            for (int k = tid; k < nv; k += NT) pdst[k] = __ldg(ps + k);
        }
    }
    __syncthreads();
    const Real* P = STAGE_P ? Ps : Pg;

    double beta;
    uint32_t sweep0;
    if (a.use_override) {
        beta = a.beta_override;
        sweep0 = a.sweep_override;
    } else {
        beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
        sweep0 = a.ctl[0] * (uint32_t)a.ptswapever;
    }
    const float kb = (float)(-2.0 * beta * 1.4426950408889634);
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    Acc acc{0, 0, 0, 0, 0};
    int* fl = (MODE == kModeSweep) ? flip_row(a, conf, rep) : nullptr;
    const CompactSpins words(reinterpret_cast<uint32_t*>(S), g);
    const FlatBytes bytes{S};

    for (int t = 0; t < a.nsweeps; ++t) {
        const uint32_t sweep = sweep0 + (uint32_t)t;
#pragma unroll 1
        for (int c = 0; c < 8; ++c) {
            if constexpr (QUAD) {
                const int nq = g.Nc >> 2;
                for (int q = tid; q < nq; q += NT)
                    quad_step<Real, MASKS, false>(a, g, words, P, BM, c, q, sweep, (uint32_t)rep,
                                                  k0, k1, beta, kb, acc, fl);
            } else {
                for (int k = tid; k < g.Nc; k += NT) {
                    const int X = k % g.Lh, r = k / g.Lh;
                    const int Y = r % g.Lh, Z = r / g.Lh;
                    site_step<Real, MASKS, MODE, false>(a, g, bytes, P, BM, Pf32, c, X, Y, Z,
                                                        sweep, (uint32_t)rep, k0, k1, beta, kb,
                                                        acc, fl);
                }
            }
            __syncthreads();
        }
    }

    if constexpr (MODE == kModeAudit) {
        Acc t = block_reduce(acc);
        if (tid == 0) {
            atomicAdd(&a.audit[0], (unsigned long long)t.M);
            atomicAdd(&a.audit[1], (unsigned long long)t.SX);
        }
        __syncthreads();
        acc = Acc{0, 0, 0, 0, 0};
    }

    // observables of the new configuration (no writes: no barrier between colours)
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
        if constexpr (QUAD) {
            const int nq = g.Nc >> 2;
            for (int q = tid; q < nq; q += NT)
                quad_step<Real, MASKS, true>(a, g, words, P, BM, c, q, 0u, 0u, 0u, 0u, beta, kb,
                                             acc);
        } else {
            for (int k = tid; k < g.Nc; k += NT) {
                const int X = k % g.Lh, r = k / g.Lh;
                const int Y = r % g.Lh, Z = r / g.Lh;
                site_step<Real, MASKS, MODE, true>(a, g, bytes, P, BM, Pf32, c, X, Y, Z, 0u, 0u,
                                                   0u, 0u, beta, kb, acc);
            }
        }
    }
    const Acc tot = block_reduce(acc);
    if (tid == 0) {
        LatObs o;
        o.eacc = tot.e;
        o.M = tot.M;
        o.SX = tot.SX;
        o.SY = tot.SY;
        o.NB = tot.NB;
        o.pad[0] = o.pad[1] = 0;
        a.obs[lat] = o;
    }
    {  // write the lattice back
        const uint4* src = reinterpret_cast<const uint4*>(S);
        uint4* dst = reinterpret_cast<uint4*>(Sg);
        for (int k = tid; k < Nb / 16; k += NT) dst[k] = src[k];
    }
}

// ------------------------------------------------------------------------------------------------
// PT swap + per-slot accumulation: one warp per conf, kSwapWarps confs per CTA.  The last CTA to
// finish (atomic ticket) advances the cycle counter and the swap phase for the next cycle.
// ------------------------------------------------------------------------------------------------
constexpr int kSwapWarps = 4;

__global__ void __launch_bounds__(32 * kSwapWarps) swap_kernel(SwapArgs a)
{
    pdl_wait();
    pdl_release();
    const uint32_t cycle = a.ctl[0];
    const int phase = (int)a.ctl[1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int conf = (int)blockIdx.x * kSwapWarps + warp;
    if (conf < a.nconf) {
        const int base = a.rbase[conf], nrep = a.nreps[conf];
        const double dn = (double)a.nocc[conf];
        const double dn1 = (double)(a.nocc[conf] < 1 ? 1 : a.nocc[conf]);
        for (int rep = lane; rep < nrep; rep += 32) {
            const LatObs o = a.obs[base + rep];
            double* lo = a.last_obs + 5 * (base + rep);
            lo[0] = (double)o.M / dn;
            lo[1] = __dmul_rn((double)o.eacc, 0x1p-33) / dn;
            lo[2] = (double)o.SX / dn;
            lo[3] = (double)o.SY / dn;
            lo[4] = (double)o.NB / dn1;
        }
        __syncwarp();
        // Pt_attempt_swaps: disjoint pairs (s, s+1), s = phase-1, phase+1, ...
        for (int s = (phase == 1 ? 0 : 1) + 2 * lane; s < nrep - 1; s += 64) {
            const int rlo = a.rat[base + s], rhi = a.rat[base + s + 1];
            a.att[base + s] += 1;
            const double elo = __dmul_rn((double)a.obs[base + rlo].eacc, 0x1p-33);
            const double ehi = __dmul_rn((double)a.obs[base + rhi].eacc, 0x1p-33);
            const double delta =
                __dmul_rn(__dsub_rn(a.beta[base + s], a.beta[base + s + 1]), __dsub_rn(elo, ehi));
            bool accept = delta >= 0.0;
            if (!accept) {
                const U4 r = philox4x32_10(cycle, (uint32_t)s, 0u, kTagSwap, a.seed,
                                           a.conf_base + (uint32_t)conf);
                accept = (double)r.x * 0x1p-32 < own_exp(delta);
            }
            if (accept) {
                a.acc[base + s] += 1;
                a.rat[base + s] = rhi;
                a.rat[base + s + 1] = rlo;
                a.tor[base + rlo] = s + 1;
                a.tor[base + rhi] = s;
            }
        }
        __syncwarp();
        if (a.measure) {
            const long long trow = a.nmeas[base];  // measured cycles so far (every slot alike)
            __syncwarp();
            const bool tracing = trow < a.trace_cap;
            for (int rep = lane; rep < nrep; rep += 32) {
                const int t = a.tor[base + rep];
                if (t == 0) a.visited[base + rep] |= 1;
                if (t == nrep - 1) a.visited[base + rep] |= 2;
                if (tracing) a.trace_tor[trow * a.entries + base + rep] = t;
            }
            for (int sl = lane; sl < nrep; sl += 32) {
                const double* o = a.last_obs + 5 * (base + a.rat[base + sl]);
                double* S = a.sums + 22 * (base + sl);
                const double amag = o[0], aen = o[1], ax = o[2], ay = o[3], anb = o[4];
                const double x2 = __dmul_rn(ax, ax), y2 = __dmul_rn(ay, ay);
                const double str2 = __dadd_rn(x2, y2);
                const double absstr = __dsqrt_rn(str2);
                const double nem = fabs(__dsub_rn(y2, x2));
                const double m2 = __dmul_rn(amag, amag), nb2 = __dmul_rn(anb, anb);
                S[0] = __dadd_rn(S[0], amag);
                S[1] = __dadd_rn(S[1], fabs(amag));
                S[2] = __dadd_rn(S[2], m2);
                S[3] = __dadd_rn(S[3], __dmul_rn(m2, m2));
                S[4] = __dadd_rn(S[4], aen);
                S[5] = __dadd_rn(S[5], __dmul_rn(aen, aen));
                S[6] = __dadd_rn(S[6], fabs(ax));
                S[7] = __dadd_rn(S[7], fabs(ay));
                S[8] = __dadd_rn(S[8], x2);
                S[9] = __dadd_rn(S[9], __dmul_rn(x2, x2));
                S[10] = __dadd_rn(S[10], y2);
                S[11] = __dadd_rn(S[11], __dmul_rn(y2, y2));
                S[12] = __dadd_rn(S[12], str2);
                S[13] = __dadd_rn(S[13], __dmul_rn(str2, str2));
                S[14] = __dadd_rn(S[14], absstr);
                S[15] = __dadd_rn(S[15], nem);
                S[16] = __dadd_rn(S[16], anb);
                S[17] = __dadd_rn(S[17], fabs(anb));
                S[18] = __dadd_rn(S[18], nb2);
                S[19] = __dadd_rn(S[19], __dmul_rn(nb2, nb2));
                if (aen < S[20]) S[20] = aen;
                S[21] = aen;
                a.nmeas[base + sl] += 1;
                if (tracing) {
                    double* tr = a.trace + 5 * (trow * a.entries + base + sl);
                    tr[0] = amag;
                    tr[1] = aen;
                    tr[2] = ax;
                    tr[3] = ay;
                    tr[4] = anb;
                }
                if (a.hist_bins > 0) {  // WRITEHIST, J:1514-1523
                    const int e = base + sl;
                    double lo = a.hist_lo[e], bs = a.hist_bs[e];
                    if (bs <= 0.0) {
                        const double w = __dadd_rn(fabs(aen), 1.0);
                        lo = __dsub_rn(aen, w);
                        bs = __ddiv_rn(__dsub_rn(__dadd_rn(aen, w), lo), (double)a.hist_bins);
                        a.hist_lo[e] = lo;
                        a.hist_bs[e] = bs;
                    }
                    int k = 1 + (int)__ddiv_rn(__dsub_rn(aen, lo), bs);
                    k = k < 1 ? 1 : (k > a.hist_bins ? a.hist_bins : k);
                    a.hist[(long long)e * a.hist_bins + k - 1] += 1;
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(&a.ctl[2], 1u);
        if (t == gridDim.x - 1) {  // every other CTA has read ctl and finished
            a.ctl[0] = cycle + 1u;
            a.ctl[1] = (uint32_t)(3 - phase);
            a.ctl[2] = 0u;
            __threadfence();
        }
    }
}

// Accumulate_local_nematic_average (J:1009-1025) on the replica at one slot of every conf of a
// group: per occupied site, s and s*(s_+x + s_-x - s_+y - s_-y) (vacant neighbours count 0).
__global__ void __launch_bounds__(256) locnem_kernel(LocnemArgs a)
{
    const Geo g = a.g;
    const int conf = (int)blockIdx.y;
    const int rep = a.rat[conf * a.nrep + a.slot];
    const uint8_t* S = a.spins + ((long long)conf * a.nrep + rep) * a.lat_stride;
    int* ls = a.loc_s + (long long)conf * a.lat_stride;
    int* ln = a.loc_n + (long long)conf * a.lat_stride;
    for (int i = (int)(blockIdx.x * blockDim.x + threadIdx.x); i < g.N;
         i += (int)(gridDim.x * blockDim.x)) {
        const int s = (int)S[i] - 1;
        if (s == 0) continue;
        const int c = i / g.Nc, k = i - c * g.Nc;
        const int X = k % g.Lh, r = k / g.Lh;
        const int Y = r % g.Lh, Z = r / g.Lh;
        const int px = c & 1, py = (c >> 1) & 1;
        const int Xp = px ? wrap_p(X, g.Lh) : X, Xm = px ? X : wrap_m(X, g.Lh);
        const int Yp = py ? wrap_p(Y, g.Lh) : Y, Ym = py ? Y : wrap_m(Y, g.Lh);
        const int nx = (int)S[cidx(g, c ^ 1, Z, Y, Xp)] + (int)S[cidx(g, c ^ 1, Z, Y, Xm)] - 2;
        const int ny = (int)S[cidx(g, c ^ 2, Z, Yp, X)] + (int)S[cidx(g, c ^ 2, Z, Ym, X)] - 2;
        ls[i] += s;
        ln[i] += s * (nx - ny);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.samples[conf] += 1;
}

// ------------------------------------------------------------------------------------------------
// Lattices too large for shared memory (L = 96: 864 KiB of spins): one launch per colour phase,
// grid (work items / CTA, lattices); the kernel boundary is the barrier between colours.  Spins
// and the field stay in HBM / L2; the measurement is a separate launch that reduces per CTA and
// adds into the (zeroed) per-lattice observables with atomics.
// ------------------------------------------------------------------------------------------------
template <class Real, bool QUAD, bool MASKS>
__global__ void __launch_bounds__(256) sweep_global_kernel(SweepArgs a, int colour, int t)
{
    pdl_wait();
    pdl_release();
    const Geo g = a.g;
    const int lat = a.lat0 + (int)blockIdx.y;
    if (a.zero_obs && blockIdx.x == 0 && threadIdx.x == 0)  // the measurement launch adds here
        store_obs(a.obs + lat, Acc{0, 0, 0, 0, 0});
    const int conf = lat / a.nrep;
    const int rep = lat - conf * a.nrep;
    uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    const Real* P = field_base<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    // FP64 reads the slot's beta, FP32 the slot's acceptance scale (rounded once from beta on
    // the host: no FP64 operation on a thread that updates one site)
    double beta = 0.0;
    float kb = 0.0f;
    uint32_t sweep;
    if (a.use_override) {
        beta = a.beta_override;
        kb = (float)(-2.0 * beta * 1.4426950408889634);
        sweep = a.sweep_override + (uint32_t)t;
    } else {
        const int slot = a.temp_of_rep[conf * a.nrep + rep];
        if constexpr (sizeof(Real) == 8)
            beta = a.beta[conf * a.nrep + slot];
        else
            kb = a.kb[conf * a.nrep + slot];
        sweep = a.ctl[0] * (uint32_t)a.ptswapever + (uint32_t)t;
    }
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    const int item = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    Acc acc{0, 0, 0, 0, 0};
    int* fl = flip_row(a, conf, rep);
    if constexpr (QUAD) {
        if (item < (g.Nc >> 2))
            quad_step<Real, MASKS, false>(a, g, CompactSpins(reinterpret_cast<uint32_t*>(S), g), P,
                                          BM, colour, item, sweep, (uint32_t)rep, k0, k1, beta,
                                          kb, acc, fl);
    } else {
        if (item < g.Nc) {
            const int X = item % g.Lh, r = item / g.Lh;
            site_step<Real, MASKS, kModeSweep, false>(a, g, FlatBytes{S}, P, BM, nullptr, colour,
                                                      X, r % g.Lh, r / g.Lh, sweep,
                                                      (uint32_t)rep, k0, k1, beta, kb, acc, fl);
        }
    }
}

template <class Real, bool QUAD, bool MASKS>
__global__ void __launch_bounds__(256) measure_global_kernel(SweepArgs a)
{
    pdl_wait();
    pdl_release();
    const Geo g = a.g;
    const int lat = a.lat0 + (int)blockIdx.y;
    const int conf = lat / a.nrep;
    uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    const Real* P = field_base<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    const int per = QUAD ? (g.Nc >> 2) : g.Nc;
    const int item = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    Acc acc{0, 0, 0, 0, 0};
    if (item < 8 * per) {
        const int c = item / per, k = item - c * per;
        if constexpr (QUAD) {
            quad_step<Real, MASKS, true>(a, g, CompactSpins(reinterpret_cast<uint32_t*>(S), g), P,
                                         BM, c, k, 0u, 0u, 0u, 0u, 0.0, 0.0f, acc);
        } else {
            const int X = k % g.Lh, r = k / g.Lh;
            site_step<Real, MASKS, kModeSweep, true>(a, g, FlatBytes{S}, P, BM, nullptr, c, X,
                                                     r % g.Lh, r / g.Lh, 0u, 0u, 0u, 0u, 0.0,
                                                     0.0f, acc);
        }
    }
    const Acc tot = block_reduce(acc);
    if (threadIdx.x == 0) {
        LatObs* o = a.obs + lat;
        atomicAdd(reinterpret_cast<unsigned long long*>(&o->eacc), (unsigned long long)tot.e);
        atomicAdd(&o->M, tot.M);
        atomicAdd(&o->SX, tot.SX);
        atomicAdd(&o->SY, tot.SY);
        atomicAdd(&o->NB, tot.NB);
    }
}

// ------------------------------------------------------------------------------------------------
// Small batches in one cooperative launch: the colour phases of the global-memory form, every
// sweep of the cycle and the observable reduction in one kernel whose CTAs are all resident (a
// cooperative launch), a grid-wide barrier between colour phases instead of a kernel boundary.
// Same per-site / per-quad arithmetic, Philox words and integer sums as the one-launch-per-colour
// form, so the results are bit for bit those of every other kernel.
// ------------------------------------------------------------------------------------------------
constexpr int kGridWait = 1 << 22;  // polls of one grid barrier before it gives up

// Grid-wide barrier: bar[0] counts arrivals, bar[1] the barriers passed (both zero at the
// launch).  Thread 0 of each CTA arrives after the CTA's barrier and a device-scope fence (which
// publishes the CTA's writes); the last arrival resets the count and releases the others, who
// wait at most kGridWait polls (a wait that gives up sets err and goes on: nothing hangs, and the
// host reports J1J2C_ETIMEOUT).
__device__ __forceinline__ void grid_barrier(unsigned* bar, unsigned nblocks, unsigned& passed,
                                             int* err)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned want = passed + 1u;
        __threadfence();
        if (atomicAdd(&bar[0], 1u) == nblocks - 1u) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicExch(&bar[1], want);
        } else {
            int it = 0;
            while (*reinterpret_cast<volatile unsigned*>(&bar[1]) != want) {
                if (++it >= kGridWait) {
                    if (err) atomicExch(err, 1);
                    break;
                }
            }
        }
        __threadfence();
        passed = want;
    }
    __syncthreads();
}

// Grid (work items / CTA, lattices), every CTA resident; bar: two zeroed words; a.obs of the
// launch's lattices zeroed before it
template <class Real, bool QUAD, bool MASKS>
__global__ void __launch_bounds__(256) sweep_coop_kernel(SweepArgs a, unsigned* bar)
{
    const Geo g = a.g;
    const int lat = a.lat0 + (int)blockIdx.y;
    const int conf = lat / a.nrep;
    const int rep = lat - conf * a.nrep;
    uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    const Real* P = field_base<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    double beta;
    uint32_t sweep0;
    if (a.use_override) {
        beta = a.beta_override;
        sweep0 = a.sweep_override;
    } else {
        beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
        sweep0 = a.ctl[0] * (uint32_t)a.ptswapever;
    }
    const float kb = (float)(-2.0 * beta * 1.4426950408889634);
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    const int item = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int per = QUAD ? (g.Nc >> 2) : g.Nc;
    const unsigned nblocks = gridDim.x * gridDim.y;
    unsigned passed = 0;
    int* fl = flip_row(a, conf, rep);
    Acc acc{0, 0, 0, 0, 0};
#pragma unroll 1
    for (int t = 0; t < a.nsweeps; ++t)
#pragma unroll 1
        for (int colour = 0; colour < 8; ++colour) {
            if (item < per) {
                const uint32_t sweep = sweep0 + (uint32_t)t;
                if constexpr (QUAD) {
                    quad_step<Real, MASKS, false>(a, g,
                                                  CompactSpins(reinterpret_cast<uint32_t*>(S), g),
                                                  P, BM, colour, item, sweep, (uint32_t)rep, k0,
                                                  k1, beta, kb, acc, fl);
                } else {
                    const int X = item % g.Lh, r = item / g.Lh;
                    site_step<Real, MASKS, kModeSweep, false>(a, g, FlatBytes{S}, P, BM, nullptr,
                                                              colour, X, r % g.Lh, r / g.Lh,
                                                              sweep, (uint32_t)rep, k0, k1, beta,
                                                              kb, acc, fl);
                }
            }
            grid_barrier(bar, nblocks, passed, a.err);
        }
    // observables: this thread's item in every colour (integer sums: any order gives the same)
    if (item < per)
#pragma unroll 1
        for (int c = 0; c < 8; ++c) {
            if constexpr (QUAD) {
                quad_step<Real, MASKS, true>(a, g,
                                             CompactSpins(reinterpret_cast<uint32_t*>(S), g), P,
                                             BM, c, item, 0u, 0u, 0u, 0u, 0.0, 0.0f, acc);
            } else {
                const int X = item % g.Lh, r = item / g.Lh;
                site_step<Real, MASKS, kModeSweep, true>(a, g, FlatBytes{S}, P, BM, nullptr, c,
                                                         X, r % g.Lh, r / g.Lh, 0u, 0u, 0u, 0u,
                                                         0.0, 0.0f, acc);
            }
        }
    const Acc tot = block_reduce(acc);
    if (threadIdx.x == 0) {
        LatObs* o = a.obs + lat;
        atomicAdd(reinterpret_cast<unsigned long long*>(&o->eacc), (unsigned long long)tot.e);
        atomicAdd(&o->M, tot.M);
        atomicAdd(&o->SX, tot.SX);
        atomicAdd(&o->SY, tot.SY);
        atomicAdd(&o->NB, tot.NB);
    }
}

// HOT (device Philox), FER, STR starts for every replica of one conf; vacancies stored as 0
__global__ void init_kernel(InitArgs a)
{
    const Geo g = a.g;
    const int rep = (int)blockIdx.y;
    uint8_t* S = a.spins + (long long)rep * a.lat_stride;
    for (int i = (int)(blockIdx.x * blockDim.x + threadIdx.x); i < g.N;
         i += (int)(gridDim.x * blockDim.x)) {
        const int c = i / g.Nc, k = i - c * g.Nc;
        const int X = k % g.Lh, r = k / g.Lh;
        const int Y = r % g.Lh, Z = r / g.Lh;
        const int x = 2 * X + (c & 1), y = 2 * Y + ((c >> 1) & 1);
        int s;
        if (a.start == 0) {
            const uint32_t grp = (uint32_t)(((c * g.Hh + Z) * g.Lh + Y) * g.Qr + (X >> 2));
            const uint32_t w =
                u4_word(philox4x32_10((uint32_t)rep, 0u, grp, kTagInit, a.seed, a.key1), X & 3);
            s = w < 0x80000000u ? 1 : -1;
        } else if (a.start == 1) {
            s = 1;
        } else {
            s = (((a.axis == 0) ? y : x) & 1) ? -1 : 1;
        }
        S[i] = a.occ[i] ? (uint8_t)(s + 1) : (uint8_t)1;
    }
}

template <class Real, bool QUAD, bool STAGE_P, bool MASKS, int MODE>
cudaError_t do_launch(const SweepArgs& a, int nblocks, int nthreads, size_t smem,
                      cudaStream_t st, bool prepare)
{
    auto k = sweep_kernel<Real, QUAD, STAGE_P, MASKS, MODE>;
    if (prepare) return raise_smem_limit(k);  // one instantiation serves every shape
    k<<<nblocks, nthreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <class Real, bool QUAD, bool STAGE_P>
cudaError_t dispatch_masks(const SweepArgs& a, const SweepVariant& v, int nb, int nt, size_t sm,
                           cudaStream_t st, bool prep)
{
    if (v.mode == kModeAudit) {
        if constexpr (sizeof(Real) == 8 && !QUAD && !STAGE_P) {
            return v.masks
                       ? do_launch<Real, false, false, true, kModeAudit>(a, nb, nt, sm, st, prep)
                       : do_launch<Real, false, false, false, kModeAudit>(a, nb, nt, sm, st, prep);
        }
        return cudaErrorInvalidValue;
    }
    return v.masks ? do_launch<Real, QUAD, STAGE_P, true, kModeSweep>(a, nb, nt, sm, st, prep)
                   : do_launch<Real, QUAD, STAGE_P, false, kModeSweep>(a, nb, nt, sm, st, prep);
}

template <class Real>
cudaError_t dispatch_shape(const SweepArgs& a, const SweepVariant& v, int nb, int nt, size_t sm,
                           cudaStream_t st, bool prep)
{
    if (v.quad)
        return v.stage_p ? dispatch_masks<Real, true, true>(a, v, nb, nt, sm, st, prep)
                         : dispatch_masks<Real, true, false>(a, v, nb, nt, sm, st, prep);
    return v.stage_p ? dispatch_masks<Real, false, true>(a, v, nb, nt, sm, st, prep)
                     : dispatch_masks<Real, false, false>(a, v, nb, nt, sm, st, prep);
}

cudaError_t dispatch(const SweepArgs& a, const SweepVariant& v, int nb, int nt, size_t sm,
                     cudaStream_t st, bool prep)
{
    return v.fp64 ? dispatch_shape<double>(a, v, nb, nt, sm, st, prep)
                  : dispatch_shape<float>(a, v, nb, nt, sm, st, prep);
}

}  // namespace

size_t sweep_smem_bytes(const Geo& g, const SweepVariant& v)
{
    const size_t spins = (size_t)((g.N + 15) & ~15);
    const size_t field = ((size_t)g.N * (v.fp64 ? 8 : 4) + 15) & ~(size_t)15;
    if (v.fixed_nt > 0 && v.stream) return field + 2 * spins;  // two spin buffers
    if (v.fixed_nt > 0 && v.rpc > 1) return field + (size_t)v.rpc * spins;  // replicas per CTA
    size_t b = spins;
    if (v.stage_p) b += (size_t)g.N * (v.fp64 ? 8 : 4);
    return (b + 15) & ~(size_t)15;
}

cudaError_t prepare_sweep_variant(const SweepVariant& v, size_t smem)
{
    SweepArgs dummy{};
    if (v.fixed_nt > 0) return cudaErrorInvalidValue;  // prepared with the shape: see api.cu
    return dispatch(dummy, v, 0, 0, smem, nullptr, true);
}

cudaError_t launch_sweep(const SweepArgs& a, const SweepVariant& v, int nblocks, int nthreads,
                         size_t smem, cudaStream_t st)
{
    if (v.fixed_nt > 0)
        return launch_fixed(a, v.fp64, v.vac,
                            FixedChoice{v.fixed_nt, v.stage_p, v.stream, v.minb,
                                        v.rpc > 1 ? v.rpc : 1},
                            nblocks, smem,
                            st, false);
    return dispatch(a, v, nblocks, nthreads, smem, st, false);
}

namespace {
template <class Real, bool QUAD, bool MASKS>
cudaError_t global_pass(const SweepArgs& a, int colour, int t, int nlat, int nt, cudaStream_t st,
                        bool measure)
{
    const int per = QUAD ? (a.g.Nc >> 2) : a.g.Nc;
    if (measure) {
        dim3 grid((unsigned)((8 * per + nt - 1) / nt), (unsigned)nlat);
        return launch_k(a.pdl != 0, grid, dim3((unsigned)nt), 0, st,
                        measure_global_kernel<Real, QUAD, MASKS>, a);
    }
    dim3 grid((unsigned)((per + nt - 1) / nt), (unsigned)nlat);
    return launch_k(a.pdl != 0, grid, dim3((unsigned)nt), 0, st,
                    sweep_global_kernel<Real, QUAD, MASKS>, a, colour, t);
}

template <class Real>
cudaError_t global_dispatch(const SweepArgs& a, const SweepVariant& v, int colour, int t,
                            int nlat, cudaStream_t st, bool measure)
{
    const int nt = v.threads > 0 ? v.threads : 256;
    if (nt > 256 || nt % 32) return cudaErrorInvalidValue;
    if (v.quad)
        return v.masks ? global_pass<Real, true, true>(a, colour, t, nlat, nt, st, measure)
                       : global_pass<Real, true, false>(a, colour, t, nlat, nt, st, measure);
    return v.masks ? global_pass<Real, false, true>(a, colour, t, nlat, nt, st, measure)
                   : global_pass<Real, false, false>(a, colour, t, nlat, nt, st, measure);
}
}  // namespace

namespace {
template <class Real, bool QUAD, bool MASKS>
cudaError_t coop_launch(const SweepArgs& a, int nlat, int nt, unsigned* bar, cudaStream_t st,
                        bool check)
{
    auto k = sweep_coop_kernel<Real, QUAD, MASKS>;
    const int per = QUAD ? (a.g.Nc >> 2) : a.g.Nc;
    const int gx = (per + nt - 1) / nt;
    if (check) {  // every CTA must be resident at once
        int dev = 0, nsm = 0, per_sm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, nt, 0);
        if (e != cudaSuccess) return e;
        return (long long)gx * nlat <= (long long)per_sm * nsm ? cudaSuccess
                                                                : cudaErrorCooperativeLaunchTooLarge;
    }
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)gx, (unsigned)nlat);
    cfg.blockDim = dim3((unsigned)nt);
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, a, bar);
}
}  // namespace

cudaError_t launch_sweep_coop(const SweepArgs& a, const SweepVariant& v, int nlat, unsigned* bar,
                              cudaStream_t st, bool check)
{
    const int nt = v.threads > 0 ? v.threads : 64;
    if (nt > 256 || nt % 32) return cudaErrorInvalidValue;
    if (v.fp64) {
        if (v.quad)
            return v.masks ? coop_launch<double, true, true>(a, nlat, nt, bar, st, check)
                           : coop_launch<double, true, false>(a, nlat, nt, bar, st, check);
        return v.masks ? coop_launch<double, false, true>(a, nlat, nt, bar, st, check)
                       : coop_launch<double, false, false>(a, nlat, nt, bar, st, check);
    }
    if (v.quad)
        return v.masks ? coop_launch<float, true, true>(a, nlat, nt, bar, st, check)
                       : coop_launch<float, true, false>(a, nlat, nt, bar, st, check);
    return v.masks ? coop_launch<float, false, true>(a, nlat, nt, bar, st, check)
                   : coop_launch<float, false, false>(a, nlat, nt, bar, st, check);
}

// ------------------------------------------------------------------------------------------------
// Lattices too large for one CTA's shared memory but not for a thread-block cluster's (L = 96:
// 864 KiB of spins over 8 CTAs of 108 KiB): CTA r of a lattice's cluster holds compact planes
// [z0, z0 + zpc) of every colour; a colour phase reads only the plane below and the plane above
// from the neighbouring CTAs' shared memory, and a cluster barrier separates the colour phases.
// All PTSWAPEVER sweeps and the observable reduction run in one launch.  The random field stays in
// global memory (L2-resident, shared by a configuration's replicas).
// ------------------------------------------------------------------------------------------------
namespace {

constexpr int kClusterThreads = 512;

struct ClusterSpins {
    uint32_t* local;     // this CTA's planes: [colour][plane][row][word]
    const uint32_t* lo;  // the CTA holding plane z0 - 1
    const uint32_t* hi;  // the CTA holding plane z0 + zpc
    int z0, zpc, Hh, rowstride, colstride, Qr;
    __device__ __forceinline__ uint32_t word(int cc, int ZZ, int YY, int qq) const
    {
        int d = ZZ - z0;
        if (d < 0) d += Hh;
        const int off = YY * Qr + qq;
        if (d < zpc) return local[cc * colstride + d * rowstride + off];
        if (d == zpc) return hi[cc * colstride + off];              // first plane above
        return lo[cc * colstride + (zpc - 1) * rowstride + off];    // last plane below
    }
    __device__ __forceinline__ void put(int cc, int ZZ, int YY, int qq, uint32_t v) const
    {
        local[cc * colstride + (ZZ - z0) * rowstride + YY * Qr + qq] = v;
    }
};

// The same planes as bytes, for one site per thread
struct ClusterBytes {
    uint8_t* local;
    const uint8_t* lo;
    const uint8_t* hi;
    int z0, zpc, Hh, Lh, plane, colstride;  // bytes per compact plane and per colour chunk
    __device__ __forceinline__ int get(int, int cc, int ZZ, int YY, int XX) const
    {
        int d = ZZ - z0;
        if (d < 0) d += Hh;
        const int off = YY * Lh + XX;
        if (d < zpc) return local[cc * colstride + d * plane + off];
        if (d == zpc) return hi[cc * colstride + off];
        return lo[cc * colstride + (zpc - 1) * plane + off];
    }
    __device__ __forceinline__ void set(int, int cc, int ZZ, int YY, int XX, uint8_t v) const
    {
        local[cc * colstride + (ZZ - z0) * plane + YY * Lh + XX] = v;
    }
};

// QUAD: four sites (one spin word) per thread per colour phase; else one site per thread, for
// small batches where a colour phase's latency is one site's arithmetic (the FP64 form)
template <class Real, bool MASKS, bool QUAD>
__global__ void __launch_bounds__(kClusterThreads, 2) sweep_cluster_kernel(SweepArgs a, int cs)
{
    extern __shared__ __align__(16) unsigned char smem[];
    cg::cluster_group cl = cg::this_cluster();
    const Geo g = a.g;
    const int rank = (int)cl.block_rank();
    const int lat = a.lat0 + (int)blockIdx.x / cs;
    const int conf = lat / a.nrep;
    const int rep = lat - conf * a.nrep;
    const int tid = (int)threadIdx.x, NT = (int)blockDim.x;
    const int zpc = g.Hh / cs, z0 = rank * zpc;
    const int plane_words = g.Lh * g.Qr;     // one word = one quad
    const int chunk_words = zpc * plane_words;  // this CTA's quads of one colour
    uint32_t* local = reinterpret_cast<uint32_t*>(smem);
    uint8_t* Sg = a.spins + (long long)lat * a.lat_stride;
    const size_t plane_bytes = (size_t)g.Lh * g.Lh;
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
        const uint4* src = reinterpret_cast<const uint4*>(Sg + (size_t)c * g.Nc + z0 * plane_bytes);
        uint4* dst = reinterpret_cast<uint4*>(local + c * chunk_words);
        for (int k = tid; k < chunk_words / 4; k += NT) dst[k] = src[k];
    }
    ClusterSpins sp;
    sp.local = local;
    sp.lo = cl.map_shared_rank(local, (rank + cs - 1) % cs);
    sp.hi = cl.map_shared_rank(local, (rank + 1) % cs);
    sp.z0 = z0;
    sp.zpc = zpc;
    sp.Hh = g.Hh;
    sp.rowstride = plane_words;
    sp.colstride = chunk_words;
    sp.Qr = g.Qr;
    ClusterBytes sb;
    sb.local = reinterpret_cast<uint8_t*>(sp.local);
    sb.lo = reinterpret_cast<const uint8_t*>(sp.lo);
    sb.hi = reinterpret_cast<const uint8_t*>(sp.hi);
    sb.z0 = z0;
    sb.zpc = zpc;
    sb.Hh = g.Hh;
    sb.Lh = g.Lh;
    sb.plane = 4 * plane_words;
    sb.colstride = 4 * chunk_words;
    const int chunk_sites = 4 * chunk_words;  // this CTA's sites of one colour
    cl.sync();

    const Real* P = field_base<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    double beta;
    uint32_t sweep0;
    if (a.use_override) {
        beta = a.beta_override;
        sweep0 = a.sweep_override;
    } else {
        beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
        sweep0 = a.ctl[0] * (uint32_t)a.ptswapever;
    }
    const float kb = (float)(-2.0 * beta * 1.4426950408889634);
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    int* fl = flip_row(a, conf, rep);
    Acc acc{0, 0, 0, 0, 0};
    const int q0 = z0 * plane_words;
    for (int t = 0; t < a.nsweeps; ++t) {
        const uint32_t sweep = sweep0 + (uint32_t)t;
#pragma unroll 1
        for (int c = 0; c < 8; ++c) {
            if constexpr (QUAD) {
                for (int lq = tid; lq < chunk_words; lq += NT)
                    quad_step<Real, MASKS, false>(a, g, sp, P, BM, c, q0 + lq, sweep,
                                                  (uint32_t)rep, k0, k1, beta, kb, acc, fl);
            } else {
                for (int ls = tid; ls < chunk_sites; ls += NT) {
                    const int X = ls % g.Lh, r = ls / g.Lh;
                    site_step<Real, MASKS, kModeSweep, false>(
                        a, g, sb, P, BM, nullptr, c, X, r % g.Lh, z0 + r / g.Lh, sweep,
                        (uint32_t)rep, k0, k1, beta, kb, acc, fl);
                }
            }
            cl.sync();
        }
    }
    // observables of the new configuration
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
        if constexpr (QUAD) {
            for (int lq = tid; lq < chunk_words; lq += NT)
                quad_step<Real, MASKS, true>(a, g, sp, P, BM, c, q0 + lq, 0u, 0u, 0u, 0u, beta,
                                             kb, acc);
        } else {
            for (int ls = tid; ls < chunk_sites; ls += NT) {
                const int X = ls % g.Lh, r = ls / g.Lh;
                site_step<Real, MASKS, kModeSweep, true>(a, g, sb, P, BM, nullptr, c, X,
                                                         r % g.Lh, z0 + r / g.Lh, 0u, 0u, 0u, 0u,
                                                         beta, kb, acc);
            }
        }
    }
    const Acc tot = block_reduce(acc);
    if (tid == 0) {
        LatObs* o = a.obs + lat;
        atomicAdd(reinterpret_cast<unsigned long long*>(&o->eacc), (unsigned long long)tot.e);
        atomicAdd(&o->M, tot.M);
        atomicAdd(&o->SX, tot.SX);
        atomicAdd(&o->SY, tot.SY);
        atomicAdd(&o->NB, tot.NB);
    }
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
        uint4* dst = reinterpret_cast<uint4*>(Sg + (size_t)c * g.Nc + z0 * plane_bytes);
        const uint4* src = reinterpret_cast<const uint4*>(local + c * chunk_words);
        for (int k = tid; k < chunk_words / 4; k += NT) dst[k] = src[k];
    }
    cl.sync();  // every CTA has finished reading its neighbours' shared memory
}

// The kernels' dynamic shared memory limit is the most the device allows, so every cluster size
// (and every shape in one context) launches whatever was probed last.
template <class Real, bool MASKS, bool QUAD>
cudaError_t cluster_prepare()
{
    cudaError_t e = raise_smem_limit(sweep_cluster_kernel<Real, MASKS, QUAD>);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(sweep_cluster_kernel<Real, MASKS, QUAD>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

template <class Real, bool MASKS, bool QUAD>
cudaError_t cluster_launch(const SweepArgs& a, int nlat, int cs, int nt, cudaStream_t st,
                           bool prepare)
{
    auto kern = sweep_cluster_kernel<Real, MASKS, QUAD>;
    const size_t smem = (size_t)a.g.N / (size_t)cs;
    cudaError_t e0 = cluster_prepare<Real, MASKS, QUAD>();
    if (prepare || e0 != cudaSuccess) return e0;
    if (nt <= 0) nt = kClusterThreads;
    if (nt > kClusterThreads || nt % 32) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nlat * cs));
    cfg.blockDim = dim3((unsigned)nt);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a, cs);
}

template <class Real, bool MASKS>
int cluster_fits(const Geo& g, int cs)
{
    auto kern = sweep_cluster_kernel<Real, MASKS, true>;
    const size_t smem = (size_t)g.N / (size_t)cs;
    if (cluster_prepare<Real, MASKS, true>() != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)cs);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return n;
}

int cluster_fits_any(const Geo& g, int cs, bool fp64, bool masks)
{
    return fp64 ? (masks ? cluster_fits<double, true>(g, cs) : cluster_fits<double, false>(g, cs))
                : (masks ? cluster_fits<float, true>(g, cs) : cluster_fits<float, false>(g, cs));
}

// ------------------------------------------------------------------------------------------------
// Small batches with the lattice replicated in every CTA of a cluster: each of a lattice's cs CTAs
// holds the whole lattice (and, where it fits, the whole random field) in its own shared memory
// and updates a fixed 1/cs of every colour class, one site per thread.  After a colour phase each
// CTA copies its updated words of that colour into the other CTAs' copies (distributed shared
// memory stores) and a cluster barrier publishes them, so every neighbour read is a local
// shared-memory load.  A CTA's copy is written by its peers only in their range of the colour
// just updated, which no CTA reads during that phase (colour c's update reads colour c only at
// its own sites).  Per-site arithmetic is site_step's and the Philox words and colour order are
// those of every other kernel, so the results are theirs bit for bit.  All PTSWAPEVER sweeps and
// the observables of a cycle run in one launch; rank 0 adds up the CTAs' sums and writes the
// lattice's observables (no zeroing first).  This is the form for a handful of FP64 lattices,
// whose colour phase must spread over many SMs (one SM's FP64 rate is ~2 FMA per clock).
// ------------------------------------------------------------------------------------------------
constexpr int kRepMaxThreads = 1024;
constexpr size_t kRepStageLimit = 200 * 1024;  // stage the field while the CTA stays below this

struct RepLayout {
    size_t field;  // byte offset of the field copy (after the spins)
    size_t sums;   // byte offset of the CTA's sums
    size_t total;
};

inline RepLayout rep_layout(const Geo& g, size_t real_size, bool stage)
{
    RepLayout l;
    l.field = ((size_t)g.N + 15) & ~(size_t)15;
    l.sums = l.field + (stage ? (((size_t)g.N * real_size + 15) & ~(size_t)15) : 0);
    l.total = l.sums + ((sizeof(Acc) + 15) & ~(size_t)15);
    return l;
}

inline bool rep_stage(const Geo& g, size_t real_size)
{
    return rep_layout(g, real_size, true).total <= kRepStageLimit;
}

// Grid: nlat * cs CTAs in clusters of cs (a lattice's CTAs form one cluster); field_off: byte
// offset of the field copy in shared memory, 0 when the field is read from global memory
template <class Real, bool MASKS>
__global__ void __launch_bounds__(kRepMaxThreads) sweep_rep_kernel(SweepArgs a, int cs,
                                                                   unsigned field_off,
                                                                   unsigned sums_off)
{
    extern __shared__ __align__(16) unsigned char smem[];
    cg::cluster_group cl = cg::this_cluster();
    const Geo g = a.g;
    const int rank = (int)cl.block_rank();
    const int lat = a.lat0 + (int)blockIdx.x / cs;
    const int conf = lat / a.nrep;
    const int rep = lat - conf * a.nrep;
    const int tid = (int)threadIdx.x, NT = (int)blockDim.x;
    uint8_t* S = smem;
    uint8_t* Sg = a.spins + (long long)lat * a.lat_stride;
    const Real* Pg = field_base<Real>(a, conf);
    block_copy16(S, Sg, g.N);  // N = 8 (L/2)^2 (H/2) is a multiple of 32
    const Real* P = Pg;
    if (field_off) {
        Real* Ps = reinterpret_cast<Real*>(smem + field_off);
        block_copy16_ldg(Ps, Pg, (int)((size_t)g.N * sizeof(Real)));
        P = Ps;
    }
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    double beta;
    uint32_t sweep0;
    if (a.use_override) {
        beta = a.beta_override;
        sweep0 = a.sweep_override;
    } else {
        beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
        sweep0 = a.ctl[0] * (uint32_t)a.ptswapever;
    }
    const float kb = (float)(-2.0 * beta * 1.4426950408889634);
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    int* fl = flip_row(a, conf, rep);
    const int per = g.Nc / cs;  // this CTA's sites of one colour (a multiple of 4, host-checked)
    const int j0 = rank * per, nw = per >> 2;
    cl.sync();  // every copy is loaded before any peer writes into it
    Acc acc{0, 0, 0, 0, 0};
#pragma unroll 1
    for (int t = 0; t < a.nsweeps; ++t) {
        const uint32_t sweep = sweep0 + (uint32_t)t;
#pragma unroll 1
        for (int c = 0; c < 8; ++c) {
            for (int k = tid; k < per; k += NT) {
                const int j = j0 + k, X = j % g.Lh, r = j / g.Lh;
                site_step<Real, MASKS, kModeSweep, false>(a, g, FlatBytes{S}, P, BM, nullptr, c,
                                                          X, r % g.Lh, r / g.Lh, sweep,
                                                          (uint32_t)rep, k0, k1, beta, kb, acc,
                                                          fl);
            }
            __syncthreads();
            uint32_t* mine = reinterpret_cast<uint32_t*>(S + (size_t)c * g.Nc + j0);
            for (int k = tid; k < (cs - 1) * nw; k += NT) {
                const int p = k / nw, w = k - p * nw;
                cl.map_shared_rank(mine, p < rank ? p : p + 1)[w] = mine[w];
            }
            cl.sync();
        }
    }
    // observables of the new configuration: this CTA's sites of every colour
    acc = Acc{0, 0, 0, 0, 0};
#pragma unroll 1
    for (int c = 0; c < 8; ++c)
        for (int k = tid; k < per; k += NT) {
            const int j = j0 + k, X = j % g.Lh, r = j / g.Lh;
            site_step<Real, MASKS, kModeSweep, true>(a, g, FlatBytes{S}, P, BM, nullptr, c, X,
                                                     r % g.Lh, r / g.Lh, 0u, 0u, 0u, 0u, beta, kb,
                                                     acc);
        }
    const Acc tot = block_reduce(acc);
    Acc* sums = reinterpret_cast<Acc*>(smem + sums_off);
    if (tid == 0) *sums = tot;
    cl.sync();
    if (rank == 0 && tid == 0) {
        Acc all{0, 0, 0, 0, 0};
        for (int p = 0; p < cs; ++p) {  // integer sums: any order gives the same
            const Acc v = *cl.map_shared_rank(sums, p);
            all.e += v.e;
            all.M += v.M;
            all.SX += v.SX;
            all.SY += v.SY;
            all.NB += v.NB;
        }
        store_obs(a.obs + lat, all);
    }
    // this CTA's range of every colour back to HBM (every copy holds the same configuration)
    for (int k = tid; k < 8 * nw; k += NT) {
        const int c = k / nw, w = k - c * nw;
        reinterpret_cast<uint32_t*>(Sg + (size_t)c * g.Nc + j0)[w] =
            reinterpret_cast<const uint32_t*>(S + (size_t)c * g.Nc + j0)[w];
    }
    cl.sync();  // rank 0 has read every CTA's sums
}

// Compile-time shape of the replicated-lattice form for the FP64 small batches (L = H = 16, 24;
// no diluted bond, no audit): a thread's site has the same position in every colour class, so
// its eleven in-class neighbour offsets (rows Y-1, Y, Y+1 times columns X-1, X, X+1, and planes
// Z+1, Z-1) and its Philox group are computed once per launch, and each colour phase only adds a
// class base that is a compile-time constant.  The arithmetic, operation for operation, is
// site_step's FP64 path (field_fp64, downhill, accept_fp64 on the same Philox word).
template <int LH, int HH>
struct RepSite {
    static constexpr int Nc = LH * LH * HH;
    static constexpr int Qr = (LH + 3) / 4;
    int off[3][3];  // [Y-1, Y, Y+1][X-1, X, X+1] within a class
    int zp, zm;     // (Z+1, Y, X) and (Z-1, Y, X)
    int g0;         // Philox group within a class
    int w;          // word of the group
    __device__ __forceinline__ explicit RepSite(int j)
    {
        const int X = j % LH, Y = (j / LH) % LH, Z = j / (LH * LH);
        const int xs[3] = {X == 0 ? LH - 1 : X - 1, X, X + 1 == LH ? 0 : X + 1};
        const int ys[3] = {Y == 0 ? LH - 1 : Y - 1, Y, Y + 1 == LH ? 0 : Y + 1};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) off[a][b] = (Z * LH + ys[a]) * LH + xs[b];
        zp = ((Z + 1 == HH ? 0 : Z + 1) * LH + Y) * LH + X;
        zm = ((Z == 0 ? HH - 1 : Z - 1) * LH + Y) * LH + X;
        g0 = (Z * LH + Y) * Qr + (X >> 2);
        w = X & 3;
    }
};

template <int LH, int HH, bool MEASURE>
__device__ __forceinline__ void rep_site(const SweepArgs& a, uint8_t* S, const double* P,
                                         const RepSite<LH, HH>& st, int C, uint32_t sweep,
                                         uint32_t rep, uint32_t k0, uint32_t k1, double beta,
                                         Acc& acc, int* fl)
{
    // one copy of the code for every colour (the fully unrolled form stalled on instruction
    // fetch with one warp per scheduler): the colour's parities select among the offsets
    constexpr int Nc = RepSite<LH, HH>::Nc;
    const bool px = C & 1, py = (C >> 1) & 1, pz = C >> 2;
    const int B0 = C * Nc, B1 = (C ^ 1) * Nc, B2 = (C ^ 2) * Nc, B3 = (C ^ 3) * Nc,
              B4 = (C ^ 4) * Nc;
    const int o = st.off[1][1];
    const int i = B0 + o;
    const int b = S[i];
    if (b == 1) return;  // vacancy: no attempt and no measured term (J:2563, J:2825)
    // the Philox word first: it does not depend on the field, so its latency overlaps the FP64
    // chain (the downhill test below decides whether it is used)
    uint32_t r = 0;
    if constexpr (!MEASURE) {
        const uint32_t grp = (uint32_t)(C * HH * LH * RepSite<LH, HH>::Qr + st.g0);
        r = u4_word(philox4x32_10(rep, sweep, grp, kTagSweep, k0, k1), st.w);
    }
    const int i1 = B2 + (py ? st.off[2][1] : o), i2 = B2 + (py ? o : st.off[0][1]);
    const int i3 = B1 + (px ? st.off[1][2] : o), i4 = B1 + (px ? o : st.off[1][0]);
    const int dpp = py ? (px ? st.off[2][2] : st.off[2][1]) : (px ? st.off[1][2] : o);
    const int dpm = py ? (px ? st.off[2][1] : st.off[2][0]) : (px ? o : st.off[1][0]);
    const int dmp = py ? (px ? st.off[1][2] : o) : (px ? st.off[0][2] : st.off[0][1]);
    const int dmm = py ? (px ? o : st.off[1][0]) : (px ? st.off[0][1] : st.off[0][0]);
    const int b1 = S[i1], b2 = S[i2], b3 = S[i3], b4 = S[i4];
    const int b5 = S[B3 + dpp], b6 = S[B3 + dpm], b7 = S[B3 + dmp], b8 = S[B3 + dmm];
    const int b9 = S[B4 + (pz ? st.zp : o)];
    const int b10 = S[B4 + (pz ? o : st.zm)];
    const int s = b - 1;
    if constexpr (MEASURE) {
        acc.M += s;
        acc.SX += px ? -s : s;
        acc.SY += py ? -s : s;
        acc.NB += s * (b3 + b4 - b1 - b2);
    }
    Nbr64 n;
    n.s[0] = b1 - 1;
    n.s[1] = b2 - 1;
    n.s[2] = b3 - 1;
    n.s[3] = b4 - 1;
    n.s[4] = b5 - 1;
    n.s[5] = b6 - 1;
    n.s[6] = b7 - 1;
    n.s[7] = b8 - 1;
    n.s[8] = b9 - 1;
    n.s[9] = b10 - 1;
    n.p1 = P[i1];
    n.p2 = P[i2];
    n.p3 = P[i3];
    n.p4 = P[i4];
    n.jv_own = n.jv_m2 = n.jh_own = n.jh_m4 = 1;
    const double f64 = field_fp64(n, P[i], a.J1h, a.J1v, a.J2, a.J3, nullptr);
    if constexpr (MEASURE) {
        acc.e += efix(spin_mul(-s, f64));
    } else {
        const bool flip = downhill(f64, s) || accept_fp64(r, metropolis_arg(f64, beta, s));
        if (flip) {
            S[i] = (uint8_t)(2 - b);
            if (fl) fl[i] += 1;
        }
    }
}

// This CTA's words of colour C (sites [j0, j0 + per) of the class) into the other CTAs' copies
template <int Nc, int CS, int NW>
__device__ __forceinline__ void rep_push(cg::cluster_group& cl, uint8_t* S, int C, int rank, int j0)
{
    uint32_t* mine = reinterpret_cast<uint32_t*>(S + C * Nc + j0);
    for (int k = (int)threadIdx.x; k < (CS - 1) * NW; k += (int)blockDim.x) {
        const int p = k / NW, w = k - p * NW;
        cl.map_shared_rank(mine, p < rank ? p : p + 1)[w] = mine[w];
    }
}

// Grid: nlat * CS CTAs of round_up(Nc / CS, 32) threads in clusters of CS; shared memory: the
// lattice, the FP64 field, the CTA's sums (rep_layout with the field staged)
template <int LH, int HH, int CS>
__global__ void __launch_bounds__(((LH * LH * HH / CS) + 31) / 32 * 32)
    sweep_rep_fixed_kernel(SweepArgs a, unsigned field_off, unsigned sums_off)
{
    constexpr int Nc = RepSite<LH, HH>::Nc, N = 8 * Nc, per = Nc / CS, NW = per / 4;
    static_assert(per % 4 == 0, "a CTA's share of a colour must be whole words");
    extern __shared__ __align__(16) unsigned char smem[];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int lat = a.lat0 + (int)blockIdx.x / CS;
    const int conf = lat / a.nrep;
    const int rep = lat - conf * a.nrep;
    const int tid = (int)threadIdx.x;
    uint8_t* S = smem;
    uint8_t* Sg = a.spins + (long long)lat * a.lat_stride;
    double* P = reinterpret_cast<double*>(smem + field_off);
    block_copy16(S, Sg, N);
    block_copy16_ldg(P, field_base<double>(a, conf), N * (int)sizeof(double));
    double beta;
    uint32_t sweep0;
    if (a.use_override) {
        beta = a.beta_override;
        sweep0 = a.sweep_override;
    } else {
        beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
        sweep0 = a.ctl[0] * (uint32_t)a.ptswapever;
    }
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    int* fl = flip_row(a, conf, rep);
    const int j0 = rank * per;
    const bool active = tid < per;
    const RepSite<LH, HH> st(j0 + (active ? tid : 0));
    cl.sync();  // every copy is loaded before any peer writes into it
    Acc acc{0, 0, 0, 0, 0};
#pragma unroll 1
    for (int t = 0; t < a.nsweeps; ++t) {
        const uint32_t sweep = sweep0 + (uint32_t)t;
#pragma unroll 1
        for (int c = 0; c < 8; ++c) {
            if (active)
                rep_site<LH, HH, false>(a, S, P, st, c, sweep, (uint32_t)rep, k0, k1, beta, acc,
                                        fl);
            __syncthreads();
            rep_push<Nc, CS, NW>(cl, S, c, rank, j0);
            cl.sync();
        }
    }
    // observables of the new configuration: this CTA's site of every colour
    if (active)
#pragma unroll 1
        for (int c = 0; c < 8; ++c)
            rep_site<LH, HH, true>(a, S, P, st, c, 0u, 0u, 0u, 0u, beta, acc, nullptr);
    const Acc tot = block_reduce(acc);
    Acc* sums = reinterpret_cast<Acc*>(smem + sums_off);
    if (tid == 0) *sums = tot;
    cl.sync();
    if (rank == 0 && tid == 0) {
        Acc all{0, 0, 0, 0, 0};
        for (int p = 0; p < CS; ++p) {  // integer sums: any order gives the same
            const Acc v = *cl.map_shared_rank(sums, p);
            all.e += v.e;
            all.M += v.M;
            all.SX += v.SX;
            all.SY += v.SY;
            all.NB += v.NB;
        }
        store_obs(a.obs + lat, all);
    }
    for (int k = tid; k < 8 * NW; k += (int)blockDim.x) {
        const int c = k / NW, w = k - c * NW;
        reinterpret_cast<uint32_t*>(Sg + c * Nc + j0)[w] =
            reinterpret_cast<const uint32_t*>(S + c * Nc + j0)[w];
    }
    cl.sync();  // rank 0 has read every CTA's sums
}

template <int LH, int HH, int CS>
cudaError_t rep_fixed_launch(const SweepArgs& a, int nlat, cudaStream_t st, bool check)
{
    auto kern = sweep_rep_fixed_kernel<LH, HH, CS>;
    constexpr int NT = ((LH * LH * HH / CS) + 31) / 32 * 32;
    const RepLayout lay = rep_layout(a.g, sizeof(double), true);
    cudaError_t e = raise_smem_limit(kern);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nlat * CS));
    cfg.blockDim = dim3((unsigned)NT);
    cfg.dynamicSmemBytes = lay.total;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)CS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (check) {
        int n = 0;
        e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
        if (e == cudaSuccess && n < 1) e = cudaErrorInvalidConfiguration;
        return e;
    }
    return cudaLaunchKernelEx(&cfg, kern, a, (unsigned)lay.field, (unsigned)lay.sums);
}

// The compile-time-shape form where it exists (returns cudaErrorNotSupported otherwise)
cudaError_t rep_fixed_dispatch(const SweepArgs& a, const SweepVariant& v, int nlat,
                               cudaStream_t st, bool check)
{
    if (!v.fp64 || v.masks || v.mode != kModeSweep || a.g.L != a.g.H)
        return cudaErrorNotSupported;
    const int L = a.g.L, cs = v.rep_cs;
#define J1J2_REP_FIXED(LL, CC)                                                                    \
    if (L == LL && cs == CC) return rep_fixed_launch<LL / 2, LL / 2, CC>(a, nlat, st, check);
    J1J2_REP_FIXED(16, 4)
    J1J2_REP_FIXED(16, 8)
    J1J2_REP_FIXED(16, 16)
    J1J2_REP_FIXED(24, 4)
    J1J2_REP_FIXED(24, 8)
    J1J2_REP_FIXED(24, 16)
#undef J1J2_REP_FIXED
    return cudaErrorNotSupported;
}

template <class Real, bool MASKS>
cudaError_t rep_launch(const SweepArgs& a, int nlat, int cs, int nt, cudaStream_t st, bool check)
{
    auto kern = sweep_rep_kernel<Real, MASKS>;
    const bool stage = rep_stage(a.g, sizeof(Real));
    const RepLayout lay = rep_layout(a.g, sizeof(Real), stage);
    if (cs < 2 || cs > 16 || a.g.Nc % (4 * cs) != 0 || nt < 32 || nt > kRepMaxThreads || nt % 32)
        return cudaErrorInvalidValue;
    cudaError_t e = raise_smem_limit(kern);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nlat * cs));
    cfg.blockDim = dim3((unsigned)nt);
    cfg.dynamicSmemBytes = lay.total;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (check) {
        int n = 0;
        e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
        if (e == cudaSuccess && n < 1) e = cudaErrorInvalidConfiguration;
        return e;
    }
    return cudaLaunchKernelEx(&cfg, kern, a, cs, stage ? (unsigned)lay.field : 0u,
                              (unsigned)lay.sums);
}

}  // namespace

// CTAs per lattice of the cluster path for a shape (0: none): the smallest of 2, 4, 8 that
// divides H/2 and keeps a CTA's planes within max_smem bytes, if such clusters can be resident.
int cluster_size_for(const Geo& g, bool fp64, bool masks, size_t max_smem)
{
    if (g.Lh % 4 != 0) return 0;
    for (const int cs : {2, 4, 8}) {
        if (g.Hh % cs != 0 || (size_t)g.N / (size_t)cs > max_smem) continue;
        if (cluster_fits_any(g, cs, fp64, masks) > 0) return cs;
    }
    return 0;
}

// Every cluster size from 2 to 16 that divides H/2 and can be resident (for small batches, where
// spreading a lattice over several SMs beats one CTA per lattice); returns the count.
int cluster_sizes(const Geo& g, bool fp64, bool masks, size_t max_smem, int* out, int cap)
{
    int n = 0;
    if (g.Lh % 4 != 0) return 0;
    for (int cs = 2; cs <= 16 && n < cap; ++cs) {
        if (g.Hh % cs != 0 || (size_t)g.N / (size_t)cs > max_smem) continue;
        if (cluster_fits_any(g, cs, fp64, masks) > 0) out[n++] = cs;
    }
    return n;
}

cudaError_t launch_sweep_cluster(const SweepArgs& a, const SweepVariant& v, int nlat,
                                 cudaStream_t st)
{
    const int cs = v.cluster, nt = v.threads;
    if (v.quad) {
        if (v.fp64)
            return v.masks ? cluster_launch<double, true, true>(a, nlat, cs, nt, st, false)
                           : cluster_launch<double, false, true>(a, nlat, cs, nt, st, false);
        return v.masks ? cluster_launch<float, true, true>(a, nlat, cs, nt, st, false)
                       : cluster_launch<float, false, true>(a, nlat, cs, nt, st, false);
    }
    if (v.fp64)
        return v.masks ? cluster_launch<double, true, false>(a, nlat, cs, nt, st, false)
                       : cluster_launch<double, false, false>(a, nlat, cs, nt, st, false);
    return v.masks ? cluster_launch<float, true, false>(a, nlat, cs, nt, st, false)
                   : cluster_launch<float, false, false>(a, nlat, cs, nt, st, false);
}

size_t rep_smem_bytes(const Geo& g, bool fp64)
{
    const size_t rs = fp64 ? sizeof(double) : sizeof(float);
    return rep_layout(g, rs, rep_stage(g, rs)).total;
}

cudaError_t launch_sweep_rep(const SweepArgs& a, const SweepVariant& v, int nlat,
                             cudaStream_t st, bool check)
{
    const cudaError_t ef = rep_fixed_dispatch(a, v, nlat, st, check);
    if (ef != cudaErrorNotSupported) return ef;
    const int cs = v.rep_cs, nt = v.threads;
    if (v.fp64)
        return v.masks ? rep_launch<double, true>(a, nlat, cs, nt, st, check)
                       : rep_launch<double, false>(a, nlat, cs, nt, st, check);
    return v.masks ? rep_launch<float, true>(a, nlat, cs, nt, st, check)
                   : rep_launch<float, false>(a, nlat, cs, nt, st, check);
}

cudaError_t launch_sweep_global(const SweepArgs& a, const SweepVariant& v, int colour, int t,
                                int nlat, cudaStream_t st)
{
    if (v.fixed_nt > 0)
        return launch_fixed_hbm(a, v.fp64, v.fixed_nt, colour, t, nlat, v.rpt, st);
    return v.fp64 ? global_dispatch<double>(a, v, colour, t, nlat, st, false)
                  : global_dispatch<float>(a, v, colour, t, nlat, st, false);
}

cudaError_t launch_measure_global(const SweepArgs& a, const SweepVariant& v, int nlat,
                                  cudaStream_t st)
{
    if (v.fixed_nt > 0) return launch_fixed_hbm(a, v.fp64, v.fixed_nt, -1, 0, nlat, v.rpt, st);
    return v.fp64 ? global_dispatch<double>(a, v, 0, 0, nlat, st, true)
                  : global_dispatch<float>(a, v, 0, 0, nlat, st, true);
}

cudaError_t launch_swap(const SwapArgs& a, cudaStream_t st, bool pdl)
{
    const int nb = (a.nconf + kSwapWarps - 1) / kSwapWarps;
    return launch_k(pdl, dim3((unsigned)nb), dim3(32u * kSwapWarps), 0, st, swap_kernel, a);
}

cudaError_t launch_locnem(const LocnemArgs& a, int nconf, cudaStream_t st)
{
    int bx = (a.g.N + 255) / 256;
    if (bx > 512) bx = 512;
    locnem_kernel<<<dim3((unsigned)bx, (unsigned)nconf), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_init(const InitArgs& a, cudaStream_t st)
{
    int bx = (a.g.N + 255) / 256;
    if (bx > 1024) bx = 1024;
    dim3 grid((unsigned)bx, (unsigned)a.nrep);
    init_kernel<<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace j1j2
