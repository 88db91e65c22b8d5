// Device building blocks of the shape-specialised sweep kernels (sweep_fixed.cu) and of the
// persistent kernel over several lattice shapes (sweep_multi.cu): compile-time lattice shapes,
// the word offsets of a spin word ("quad": four sites of one compact row) and its neighbours,
// operand loads, the per-quad update and measurement of both precisions, and the eight colour
// phases of a sweep over one lattice or over R replicas of one configuration.
#pragma once
#include "sweep_common.cuh"

namespace j1j2 {
namespace {

template <int LH, int HH>
struct Shape {
    static constexpr int QR = LH / 4;    // 32-bit words per compact row
    static constexpr int RS = LH * QR;   // words per compact z-plane
    static constexpr int CS = HH * RS;   // words (= quads) per colour
    static constexpr int N = 8 * LH * LH * HH;
    static constexpr int NB = (N + 15) & ~15;
};

// Word offsets (within a colour block) of a quad and of the words its neighbours live in:
// same row; row Y+1 / Y-1; plane Z+1 / Z-1; and the words one step along x in those rows.
struct QuadOff {
    int self, xp, xm;          // row Y:   words qx, qx+1, qx-1
    int yp, yp_xp, yp_xm;      // row Y+1: words qx, qx+1, qx-1
    int ym, ym_xp, ym_xm;      // row Y-1
    int zp, zm;                // planes Z+1 / Z-1, word qx
};

template <int LH, int HH>
__device__ __forceinline__ QuadOff quad_offsets(int q)
{
    using Sh = Shape<LH, HH>;
    const int qx = q % Sh::QR, row = q / Sh::QR;
    const int Y = row % LH, Z = row / LH;
    const int qxp = qx + 1 == Sh::QR ? 0 : qx + 1, qxm = qx == 0 ? Sh::QR - 1 : qx - 1;
    const int Yp = Y + 1 == LH ? 0 : Y + 1, Ym = Y == 0 ? LH - 1 : Y - 1;
    const int Zp = Z + 1 == HH ? 0 : Z + 1, Zm = Z == 0 ? HH - 1 : Z - 1;
    const int r0 = Z * Sh::RS + Y * Sh::QR, rp = Z * Sh::RS + Yp * Sh::QR,
              rm = Z * Sh::RS + Ym * Sh::QR;
    QuadOff o;
    o.self = r0 + qx;
    o.xp = r0 + qxp;
    o.xm = r0 + qxm;
    o.yp = rp + qx;
    o.yp_xp = rp + qxp;
    o.yp_xm = rp + qxm;
    o.ym = rm + qx;
    o.ym_xp = rm + qxp;
    o.ym_xm = rm + qxm;
    o.zp = Zp * Sh::RS + Y * Sh::QR + qx;
    o.zm = Zm * Sh::RS + Y * Sh::QR + qx;
    return o;
}

// Operands of one quad in one colour phase
template <class Real>
struct QuadData {
    int self;                                    // word offset of the quad in its colour block
    uint32_t own, wxp, wxm, wyp, wym;            // spins: own, +-x, +-y
    uint32_t wdpp, wdpm, wdmp, wdmm, wzp, wzm;   // diagonals (+x+y, -x+y, +x-y, -x-y), +-z
    Real pown[4], pxa[4], pyp[4], pym[4], pextra;
};

// Neighbour rows of a quad for colour C's parities (J:540-584): odd parity steps +1, even -1
template <int C>
struct QuadRows {
    int yp, ym, xn, yp_n, ym_n, zp, zm;
    __device__ __forceinline__ explicit QuadRows(const QuadOff& o)
    {
        constexpr int px = C & 1, py = (C >> 1) & 1, pz = C >> 2;
        yp = py ? o.yp : o.self;  // +y / -y rows, word qx
        ym = py ? o.self : o.ym;
        xn = px ? o.xp : o.xm;    // same row, shifted word
        yp_n = py ? (px ? o.yp_xp : o.yp_xm) : xn;
        ym_n = py ? xn : (px ? o.ym_xp : o.ym_xm);
        zp = pz ? o.zp : o.self;
        zm = pz ? o.self : o.zm;
    }
};

// Spin words of a quad and its neighbours
template <class Real, int LH, int HH, int C>
__device__ __forceinline__ void load_quad_spins(const uint32_t* S32, const QuadOff& o,
                                                QuadData<Real>& d)
{
    using Sh = Shape<LH, HH>;
    constexpr int px = C & 1;
    constexpr int B0 = C * Sh::CS, B1 = (C ^ 1) * Sh::CS, B2 = (C ^ 2) * Sh::CS;
    constexpr int B3 = (C ^ 3) * Sh::CS, B4 = (C ^ 4) * Sh::CS;
    const QuadRows<C> r(o);
    d.self = o.self;
    d.own = S32[B0 + o.self];
    x_pair(px, S32[B1 + o.self], S32[B1 + r.xn], d.wxp, d.wxm);
    d.wyp = S32[B2 + r.yp];
    d.wym = S32[B2 + r.ym];
    x_pair(px, S32[B3 + r.yp], S32[B3 + r.yp_n], d.wdpp, d.wdpm);
    x_pair(px, S32[B3 + r.ym], S32[B3 + r.ym_n], d.wdmp, d.wdmm);
    d.wzp = S32[B4 + r.zp];
    d.wzm = S32[B4 + r.zm];
}

// Random-field values of a quad and of its +-x and +-y neighbours
template <class Real, int LH, int HH, int C>
__device__ __forceinline__ void load_quad_field(const Real* P, const QuadOff& o,
                                                QuadData<Real>& d)
{
    using Sh = Shape<LH, HH>;
    constexpr int px = C & 1;
    constexpr int B0 = C * Sh::CS, B1 = (C ^ 1) * Sh::CS, B2 = (C ^ 2) * Sh::CS;
    const QuadRows<C> r(o);
    d.pextra = P[4 * (B1 + r.xn) + (px ? 0 : 3)];
    if constexpr (sizeof(Real) == 4) {
        const float4* P4 = reinterpret_cast<const float4*>(P);
        const float4 v0 = P4[B0 + o.self], v1 = P4[B1 + o.self];
        const float4 v2 = P4[B2 + r.yp], v3 = P4[B2 + r.ym];
        d.pown[0] = v0.x, d.pown[1] = v0.y, d.pown[2] = v0.z, d.pown[3] = v0.w;
        d.pxa[0] = v1.x, d.pxa[1] = v1.y, d.pxa[2] = v1.z, d.pxa[3] = v1.w;
        d.pyp[0] = v2.x, d.pyp[1] = v2.y, d.pyp[2] = v2.z, d.pyp[3] = v2.w;
        d.pym[0] = v3.x, d.pym[1] = v3.y, d.pym[2] = v3.z, d.pym[3] = v3.w;
    } else {
        const double2* P2 = reinterpret_cast<const double2*>(P);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const double2 v0 = P2[2 * (B0 + o.self) + h], v1 = P2[2 * (B1 + o.self) + h];
            const double2 v2 = P2[2 * (B2 + r.yp) + h], v3 = P2[2 * (B2 + r.ym) + h];
            d.pown[2 * h] = v0.x, d.pown[2 * h + 1] = v0.y;
            d.pxa[2 * h] = v1.x, d.pxa[2 * h + 1] = v1.y;
            d.pyp[2 * h] = v2.x, d.pyp[2 * h + 1] = v2.y;
            d.pym[2 * h] = v3.x, d.pym[2 * h + 1] = v3.y;
        }
    }
}

template <class Real, int LH, int HH, int C>
__device__ __forceinline__ QuadData<Real> load_quad(const uint32_t* S32, const Real* P,
                                                    const QuadOff& o)
{
    QuadData<Real> d;
    load_quad_spins<Real, LH, HH, C>(S32, o, d);
    load_quad_field<Real, LH, HH, C>(P, o, d);
    return d;
}

// Byte k of the result is 0xFF when element k of the site pairs (d01: sites 0, 1; d23: sites 2, 3)
// has its sign bit set, else 0 (prmt with sign replication of each source word's top byte).
__device__ __forceinline__ uint32_t sign_bytes(f2 d01, f2 d23)
{
    uint32_t r;
    asm("{\n\t.reg .b32 a0, a1, b0, b1, m0, m1;\n\t"
        "mov.b64 {a0, a1}, %1;\n\t"
        "mov.b64 {b0, b1}, %2;\n\t"
        "prmt.b32 m0, a0, a1, 0x00FB;\n\t"
        "prmt.b32 m1, b0, b1, 0xFB00;\n\t"
        "lop3.b32 %0, m0, m1, 0x0000FFFF, 0xE4;\n\t}"
        : "=r"(r)
        : "l"(d01), "l"(d23));
    return r;
}

// Update (or measure) one quad from its loaded operands.  VAC: vacancies may be present (the
// FP32 acceptance threshold is then scaled by s^2 so that a vacancy never flips).
// qshift: words between S32 and the lattice's first word (the quad's Philox group is its
// position in the lattice); conf: the lattice's configuration within the launch (Philox key word
// 1 is conf_base + conf).  GSTORE: S32 is in global memory, where the quad's word is written
// only when a site flips; in shared memory it is always written (cheaper than the test).
template <class Real, int LH, int HH, int C, bool MEASURE, bool VAC, bool GSTORE = false>
__device__ __forceinline__ void compute_quad(const SweepArgs& a, uint32_t* S32,
                                             const QuadData<Real>& d, uint32_t sweep,
                                             uint32_t rep, uint32_t conf, double beta, float kb,
                                             Acc& acc, int qshift = 0)
{
    using Sh = Shape<LH, HH>;
    constexpr int px = C & 1, py = (C >> 1) & 1;
    constexpr int B0 = C * Sh::CS;
    U4 rnd{0, 0, 0, 0};
    if constexpr (!MEASURE) {
        const uint32_t grp = (uint32_t)(B0 + d.self + qshift);
        // shared-memory kernels: round keys from the parameters (fewer integer instructions);
        // the HBM kernels keep the plain form, which their register budget holds without spills
        if constexpr (GSTORE)
            rnd = philox4x32_10(rep, sweep, grp, kTagSweep, a.seed, a.conf_base + conf);
        else
            rnd = philox4x32_10_rk(rep, sweep, grp, kTagSweep, a.rk0, a.rk1, conf);
    }
    uint32_t flipmask = 0;
    if constexpr (sizeof(Real) == 4) {
        // Sites in pairs (0,1), (2,3) with packed FP32x2 arithmetic: every element follows
        // field_fp32's operations and rounding (the -y terms enter as products with the negated
        // spins, the J1v term as (pi - J1v) * (-sy): the same products, exactly).  The FP32
        // kernels here run only with integer J2, J3 (|J| <= 8; the host checks): the first two
        // terms, J3*Zs rounded and then fma(J2, D, .), are then an exact small integer, formed
        // for all four sites at once in integer arithmetic on the byte sums (each byte lane
        // J3*z + J2*d + bias stays in 0..255, so the word is exact modulo 2^32 lane by lane) and
        // read out of the bytes like the spins.  (A zero may differ in sign from the
        // floating-point form's, which no later sum, product or test can see.)
        const uint32_t dsum = d.wdpp + d.wdpm + d.wdmp + d.wdmm;  // bytewise, <= 8
        const uint32_t zsum = d.wzp + d.wzm;                      // bytewise, <= 4
        const uint32_t cpl = zsum * (uint32_t)a.J3i + dsum * (uint32_t)a.J2i + a.ij_bias;
        const f2 c1 = f2_splat(8388609.0f), coff = f2_splat(a.ij_off);
        const f2 j1h = f2_splat(a.J1hf), j1v = f2_splat(a.J1vf);
        int ehi = 0, elo = 0;  // fixed-point energy of the quad, split as in efix32_split
        float nbf = 0.0f;      // nematic sum of the quad (exact small integers)
        f2 dlt[2];             // u - threshold per site pair: its sign bit is the decision
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * h;
            const f2 sxp = f2_sub(byte_pair(d.wxp, k), c1);
            const f2 sxm = f2_sub(byte_pair(d.wxm, k), c1);
            const f2 nsyp = f2_sub(c1, byte_pair(d.wyp, k));   // -s at +y
            const f2 nsym = f2_sub(c1, byte_pair(d.wym, k));   // -s at -y
            const f2 si = f2_sub(byte_pair(d.own, k), c1);
            const f2 pi = f2_pack(d.pown[k], d.pown[k + 1]);
            const f2 pxp = px ? f2_pack(d.pxa[k + 1], k + 1 < 3 ? d.pxa[k + 2] : d.pextra)
                              : f2_pack(d.pxa[k], d.pxa[k + 1]);
            const f2 pxm = px ? f2_pack(d.pxa[k], d.pxa[k + 1])
                              : f2_pack(k > 0 ? d.pxa[k - 1] : d.pextra, d.pxa[k]);
            const f2 pyp = f2_pack(d.pyp[k], d.pyp[k + 1]);
            const f2 pym = f2_pack(d.pym[k], d.pym[k + 1]);
            const f2 sx = f2_add(sxp, sxm), nsy = f2_add(nsyp, nsym);
            f2 f = f2_sub(byte_pair(cpl, k), coff);  // J3*Zs + J2*D, exact
            f = f2_fma(f2_add(j1h, pi), sx, f);
            f = f2_fma(f2_sub(pi, j1v), nsy, f);
            f = f2_fma(pxp, sxp, f);
            f = f2_fma(pxm, sxm, f);
            f = f2_fma(pyp, nsyp, f);
            f = f2_fma(pym, nsym, f);
            const f2 sf = f2_mul(si, f);
            if constexpr (MEASURE) {
                const f2 x2 = f2_mul(sf, f2_splat(-65536.0f));
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const float x = f2_get(x2, e);
                    const float t = truncf(x);
                    ehi += __float2int_rz(t);
                    elo += __float2int_rn(__fmul_rn(__fsub_rn(x, t), 65536.0f));
                }
                const f2 nb = f2_mul(si, f2_add(sx, nsy));
                nbf = __fadd_rn(__fadd_rn(nbf, f2_get(nb, 0)), f2_get(nb, 1));
            } else {
                // Metropolis test u < exp(-beta dE) as 2^(kb s f); with vacancies the threshold
                // is scaled by s^2, so a vacancy (s = 0) never flips.  u < thr exactly when
                // u - thr is negative: the difference of two floats is zero only when they are
                // equal (+0 then), and u (0 or >= 2^-23) and thr (0 or normal: ex2.approx.ftz)
                // leave no room for an underflow
                const f2 arg = f2_mul(f2_splat(kb), sf);
                f2 thr = f2_pack(ex2_approx(f2_get(arg, 0)), ex2_approx(f2_get(arg, 1)));
                if constexpr (VAC) thr = f2_mul(thr, f2_mul(si, si));
                const f2 u = f2_sub(
                    f2_pack(__uint_as_float(0x3F800000u | (u4_word(rnd, k) & 0x007FFFFFu)),
                            __uint_as_float(0x3F800000u | (u4_word(rnd, k + 1) & 0x007FFFFFu))),
                    f2_splat(1.0f));
                dlt[h] = f2_sub(u, thr);
            }
        }
        if constexpr (!MEASURE) flipmask = sign_bytes(dlt[0], dlt[1]) & 0x02020202u;
        if constexpr (MEASURE) {
            // magnetisation and stripe sums from the byte sum of the own word (s = b - 1)
            const int mq = (int)((d.own * 0x01010101u) >> 24) - 4;
            acc.M += mq;
            acc.SX += px ? -mq : mq;
            acc.SY += py ? -mq : mq;
            acc.NB += (int)nbf;
            acc.e += ((long long)ehi << 16) + (long long)elo;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int sh = 8 * k;
            const int b = (d.own >> sh) & 0xFF;
            if (b == 1) continue;
            Nbr64 nb;
            nb.s[0] = (int)((d.wyp >> sh) & 0xFF) - 1;
            nb.s[1] = (int)((d.wym >> sh) & 0xFF) - 1;
            nb.s[2] = (int)((d.wxp >> sh) & 0xFF) - 1;
            nb.s[3] = (int)((d.wxm >> sh) & 0xFF) - 1;
            nb.s[4] = (int)((d.wdpp >> sh) & 0xFF) - 1;
            nb.s[5] = (int)((d.wdpm >> sh) & 0xFF) - 1;
            nb.s[6] = (int)((d.wdmp >> sh) & 0xFF) - 1;
            nb.s[7] = (int)((d.wdmm >> sh) & 0xFF) - 1;
            nb.s[8] = (int)((d.wzp >> sh) & 0xFF) - 1;
            nb.s[9] = (int)((d.wzm >> sh) & 0xFF) - 1;
            nb.p1 = d.pyp[k];
            nb.p2 = d.pym[k];
            nb.p3 = px ? (k < 3 ? d.pxa[k + 1] : d.pextra) : d.pxa[k];
            nb.p4 = px ? d.pxa[k] : (k > 0 ? d.pxa[k - 1] : d.pextra);
            nb.jv_own = nb.jv_m2 = nb.jh_own = nb.jh_m4 = 1;
            const double f = field_fp64(nb, d.pown[k], a.J1h, a.J1v, a.J2, a.J3, nullptr);
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
        if constexpr (GSTORE) {
            if (flipmask) S32[B0 + d.self] = d.own ^ flipmask;
        } else {
            S32[B0 + d.self] = d.own ^ flipmask;
        }
    }
}

// Offsets are held in registers for the whole kernel when a thread owns at most two quads;
// with more quads they are recomputed in every phase (a few constant-divisor operations) to keep
// register pressure down.
template <int QPT>
struct OffsetCache {
    static constexpr bool kHold = QPT <= 2;
    QuadOff off[kHold ? QPT : 1];
    QuadOff base;  // plane-strided threads: the first quad's offsets
    int zp_last;   // and the +z plane offset of the last quad (the only one that can wrap)
};

// A thread's quads lie NT / RS planes apart in the same row and column when NT is a whole
// number of planes and the quads exactly fill the colour: their offsets are the first quad's
// shifted by a constant, apart from the -z plane of the first and the +z plane of the last
// (periodic wrap), so nothing is recomputed per colour phase.
template <int LH, int HH, int NT, int QPT>
struct Strided {
    static constexpr int RS = Shape<LH, HH>::RS;
    static constexpr int ZS = NT / RS;  // planes between a thread's quads
    static constexpr bool value =
        QPT > 2 && NT % RS == 0 && QPT * NT == Shape<LH, HH>::CS && QPT * ZS == HH;
};

template <int LH, int HH, int NT, int QPT>
__device__ __forceinline__ void fill_offsets(OffsetCache<QPT>& off, int tid)
{
    using Sh = Shape<LH, HH>;
    if constexpr (OffsetCache<QPT>::kHold) {
#pragma unroll
        for (int j = 0; j < QPT; ++j) {
            const int q = tid + j * NT;
            off.off[j] = quad_offsets<LH, HH>(q < Sh::CS ? q : 0);
        }
    } else if constexpr (Strided<LH, HH, NT, QPT>::value) {
        off.base = quad_offsets<LH, HH>(tid);
        off.zp_last = quad_offsets<LH, HH>(tid + (QPT - 1) * NT).zp;
    }
}

template <int LH, int HH, int NT, int QPT>
__device__ __forceinline__ QuadOff offsets_for(const OffsetCache<QPT>& oc, int j)
{
    if constexpr (OffsetCache<QPT>::kHold) {
        return oc.off[j];
    } else {
        int tid;  // opaque read: stops the per-phase arithmetic from being hoisted and kept live
        asm volatile("mov.u32 %0, %%tid.x;" : "=r"(tid));
        const int q = tid + j * NT;
        return quad_offsets<LH, HH>(q < Shape<LH, HH>::CS ? q : 0);
    }
}

template <class Real, int LH, int HH, int NT, int QPT, int C, bool MEASURE, bool VAC>
__device__ __forceinline__ void colour_phase(const SweepArgs& a, uint32_t* S32, const Real* P,
                                             const OffsetCache<QPT>& oc, uint32_t sweep,
                                             uint32_t rep, uint32_t kconf, double beta,
                                             float kb, Acc& acc)
{
    constexpr int NQ = Shape<LH, HH>::CS;
    if constexpr (QPT == 2) {
        // both quads' loads first, then both updates (same-colour quads are independent)
        const bool has1 = 2 * NT == NQ || (int)threadIdx.x + NT < NQ;
        const QuadData<Real> d0 = load_quad<Real, LH, HH, C>(S32, P, oc.off[0]);
        QuadData<Real> d1 = d0;
        if (has1) d1 = load_quad<Real, LH, HH, C>(S32, P, oc.off[1]);
        compute_quad<Real, LH, HH, C, MEASURE, VAC>(a, S32, d0, sweep, rep, kconf, beta, kb,
                                                    acc);
        if (has1)
            compute_quad<Real, LH, HH, C, MEASURE, VAC>(a, S32, d1, sweep, rep, kconf, beta,
                                                        kb, acc);
    } else if constexpr (Strided<LH, HH, NT, QPT>::value) {
        constexpr int RS = Strided<LH, HH, NT, QPT>::RS;
        constexpr int SH = Strided<LH, HH, NT, QPT>::ZS * RS;  // words between the quads
#pragma unroll 2
        for (int j = 0; j < QPT; ++j) {
            const int shift = j * SH;
            QuadOff o = oc.base;
            o.zm = j == 0 ? oc.base.zm : oc.base.self - RS;
            o.zp = j == QPT - 1 ? oc.zp_last - shift : oc.base.self + RS;
            const QuadData<Real> dj = load_quad<Real, LH, HH, C>(S32 + shift, P + 4 * shift, o);
            compute_quad<Real, LH, HH, C, MEASURE, VAC>(a, S32 + shift, dj, sweep, rep, kconf,
                                                        beta, kb, acc, shift);
        }
    } else {
#pragma unroll 2
        for (int j = 0; j < QPT; ++j)
            if (QPT * NT == NQ || (int)threadIdx.x + j * NT < NQ) {
                const QuadData<Real> dj =
                    load_quad<Real, LH, HH, C>(S32, P, offsets_for<LH, HH, NT, QPT>(oc, j));
                compute_quad<Real, LH, HH, C, MEASURE, VAC>(a, S32, dj, sweep, rep, kconf,
                                                            beta, kb, acc);
            }
    }
}

template <class Real, int LH, int HH, int NT, int QPT, bool MEASURE, bool VAC>
__device__ __forceinline__ void all_colours(const SweepArgs& a, uint32_t* S32, const Real* P,
                                            const OffsetCache<QPT>& oc, uint32_t sweep,
                                            uint32_t rep, uint32_t kconf, double beta,
                                            float kb, Acc& acc)
{
    // One barrier per colour.  The measurement only reads, but without the barrier the
    // instruction scheduler interleaves all eight read-only phases and runs out of registers.
#define J1J2_PHASE(C)                                                                        \
    colour_phase<Real, LH, HH, NT, QPT, C, MEASURE, VAC>(a, S32, P, oc, sweep, rep, kconf,  \
                                                         beta, kb, acc);                     \
    __syncthreads();
    J1J2_PHASE(0)
    J1J2_PHASE(1)
    J1J2_PHASE(2)
    J1J2_PHASE(3)
    J1J2_PHASE(4)
    J1J2_PHASE(5)
    J1J2_PHASE(6)
    J1J2_PHASE(7)
#undef J1J2_PHASE
}

// Colour phases over R replicas of one configuration per CTA: their lattices side by side in
// shared memory behind one staged copy of their configuration's field.  A thread takes the same
// quad positions in all R lattices: the field operands of a position (and the arithmetic on
// them alone) are loaded once for the R quads, every replica's spin words are loaded before any
// is updated, and the lattices of a CTA share its barriers and set-up.  Results are those of
// the one-lattice form bit for bit (same operations per quad, same Philox words).
// active: the thread takes part in the colour phases (threads beyond the NT that cover a
// colour only meet the barriers).  One replica with a thread's quads one plane-stride apart
// (Strided) takes the first quad's offsets, shifted, as colour_phase does.
template <class Real, int LH, int HH, int NT, int QPT, int R, int C, bool MEASURE, bool VAC>
__device__ __forceinline__ void colour_phase_r(const SweepArgs& a, uint32_t* const (&S32)[R],
                                               const Real* P, const OffsetCache<QPT>& oc,
                                               uint32_t sweep, const int (&rep)[R],
                                               uint32_t kconf, const double (&beta)[R],
                                               const float (&kb)[R], Acc (&acc)[R], bool active)
{
    constexpr int NQ = Shape<LH, HH>::CS;
    if (!active) return;
    if constexpr (R == 1 && Strided<LH, HH, NT, QPT>::value) {
        constexpr int RS = Strided<LH, HH, NT, QPT>::RS;
        constexpr int SH = Strided<LH, HH, NT, QPT>::ZS * RS;  // words between the quads
#pragma unroll 2
        for (int j = 0; j < QPT; ++j) {
            const int shift = j * SH;
            QuadOff o = oc.base;
            o.zm = j == 0 ? oc.base.zm : oc.base.self - RS;
            o.zp = j == QPT - 1 ? oc.zp_last - shift : oc.base.self + RS;
            const QuadData<Real> dj =
                load_quad<Real, LH, HH, C>(S32[0] + shift, P + 4 * shift, o);
            compute_quad<Real, LH, HH, C, MEASURE, VAC>(a, S32[0] + shift, dj, sweep,
                                                        (uint32_t)rep[0], kconf, beta[0], kb[0],
                                                        acc[0], shift);
        }
    } else {
#pragma unroll
        for (int j = 0; j < QPT; ++j) {
            if (!(QPT * NT == NQ || (int)threadIdx.x + j * NT < NQ)) continue;
            const QuadOff o = offsets_for<LH, HH, NT, QPT>(oc, j);
            QuadData<Real> d[R];
            load_quad_field<Real, LH, HH, C>(P, o, d[0]);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r > 0) d[r] = d[0];
                load_quad_spins<Real, LH, HH, C>(S32[r], o, d[r]);
            }
#pragma unroll
            for (int r = 0; r < R; ++r)
                compute_quad<Real, LH, HH, C, MEASURE, VAC>(a, S32[r], d[r], sweep,
                                                            (uint32_t)rep[r], kconf, beta[r],
                                                            kb[r], acc[r]);
        }
    }
}

template <class Real, int LH, int HH, int NT, int QPT, int R, bool MEASURE, bool VAC>
__device__ __forceinline__ void all_colours_r(const SweepArgs& a, uint32_t* const (&S32)[R],
                                              const Real* P, const OffsetCache<QPT>& oc,
                                              uint32_t sweep, const int (&rep)[R], uint32_t kconf,
                                              const double (&beta)[R], const float (&kb)[R],
                                              Acc (&acc)[R], bool active = true)
{
#define J1J2_PHASE_R(C)                                                                       \
    colour_phase_r<Real, LH, HH, NT, QPT, R, C, MEASURE, VAC>(a, S32, P, oc, sweep, rep, kconf, \
                                                              beta, kb, acc, active);          \
    __syncthreads();
    J1J2_PHASE_R(0)
    J1J2_PHASE_R(1)
    J1J2_PHASE_R(2)
    J1J2_PHASE_R(3)
    J1J2_PHASE_R(4)
    J1J2_PHASE_R(5)
    J1J2_PHASE_R(6)
    J1J2_PHASE_R(7)
#undef J1J2_PHASE_R
}

}  // namespace
}  // namespace j1j2
