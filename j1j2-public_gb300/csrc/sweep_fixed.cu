// Shape-specialised sweep kernel: the lattice extents (L/2, H/2) and the CTA size are template
// constants and the eight colour phases of a sweep are unrolled, so colour parities are
// compile-time.  Each thread owns the same quad(s) in every colour class; the word offsets of the
// quad's neighbours inside a colour block are computed once, and a colour phase addresses shared
// memory as [offset + colour base], the base being an immediate.  With two quads per thread both
// quads' operands are loaded before either is updated (quads of one colour never neighbour each
// other), which doubles the instruction-level parallelism of a thread.  Same arithmetic, Philox
// stream and outputs as the generic quad kernel (kernels.cu), bit for bit.  One CTA owns one
// lattice, staged in shared memory for the PTSWAPEVER fused sweeps of a PT cycle.
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

template <class Real, int LH, int HH, int NT, int MINB, bool STAGE_P, bool VAC>
__global__ void __launch_bounds__(NT, MINB) sweep_fixed_kernel(SweepArgs a)
{
    using Sh = Shape<LH, HH>;
    constexpr int QPT = (Sh::CS + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lat = a.lat0 + (int)blockIdx.x;
    const int conf = lat / a.nrep;
    const int rep = lat - conf * a.nrep;
    uint8_t* S = smem;
    Real* Ps = reinterpret_cast<Real*>(smem + Sh::NB);
    uint8_t* Sg = a.spins + (long long)lat * a.lat_stride;
    const Real* Pg = field_base<Real>(a, conf);

    block_copy16(S, Sg, Sh::NB);
    if constexpr (STAGE_P)
        block_copy16_ldg(Ps, Pg, (int)((Sh::N * sizeof(Real) + 15) & ~(size_t)15));
    OffsetCache<QPT> off;
    fill_offsets<LH, HH, NT, QPT>(off, (int)threadIdx.x);
    __syncthreads();
    const Real* P = STAGE_P ? Ps : Pg;
    uint32_t* S32 = reinterpret_cast<uint32_t*>(S);

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
    const uint32_t kconf = (uint32_t)conf;
    Acc acc{0, 0, 0, 0, 0};
#pragma unroll 1
    for (int t = 0; t < a.nsweeps; ++t)
        all_colours<Real, LH, HH, NT, QPT, false, VAC>(a, S32, P, off, sweep0 + (uint32_t)t,
                                                       (uint32_t)rep, kconf, beta, kb, acc);
    all_colours<Real, LH, HH, NT, QPT, true, VAC>(a, S32, P, off, 0u, 0u, 0u, beta, kb, acc);
    const Acc tot = block_reduce(acc);
    if (threadIdx.x == 0) store_obs(a.obs + lat, tot);
    block_copy16(Sg, S, Sh::NB);
}

// The same kernel over R replicas of one configuration per CTA: their lattices side by side in
// shared memory behind one staged copy of their configuration's field.  A thread takes the same
// quad positions in all R lattices: the field operands of a position (and the arithmetic on
// them alone) are loaded once for the R quads, every replica's spin words are loaded before any
// is updated, and the lattices of a CTA share its barriers and set-up.  Results are those of
// sweep_fixed_kernel bit for bit (same operations per quad, same Philox words).
template <class Real, int LH, int HH, int NT, int QPT, int R, int C, bool MEASURE, bool VAC>
__device__ __forceinline__ void colour_phase_r(const SweepArgs& a, uint32_t* const (&S32)[R],
                                               const Real* P, const OffsetCache<QPT>& oc,
                                               uint32_t sweep, const int (&rep)[R],
                                               uint32_t kconf, const double (&beta)[R],
                                               const float (&kb)[R], Acc (&acc)[R])
{
    constexpr int NQ = Shape<LH, HH>::CS;
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
            compute_quad<Real, LH, HH, C, MEASURE, VAC>(a, S32[r], d[r], sweep, (uint32_t)rep[r],
                                                        kconf, beta[r], kb[r], acc[r]);
    }
}

template <class Real, int LH, int HH, int NT, int QPT, int R, bool MEASURE, bool VAC>
__device__ __forceinline__ void all_colours_r(const SweepArgs& a, uint32_t* const (&S32)[R],
                                              const Real* P, const OffsetCache<QPT>& oc,
                                              uint32_t sweep, const int (&rep)[R], uint32_t kconf,
                                              const double (&beta)[R], const float (&kb)[R],
                                              Acc (&acc)[R])
{
#define J1J2_PHASE_R(C)                                                                       \
    colour_phase_r<Real, LH, HH, NT, QPT, R, C, MEASURE, VAC>(a, S32, P, oc, sweep, rep, kconf, \
                                                              beta, kb, acc);                  \
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

// Grid: one CTA per R consecutive lattices from a.lat0 (the launcher guarantees that they are
// replicas of one configuration)
template <class Real, int LH, int HH, int NT, int MINB, bool VAC, int R>
__global__ void __launch_bounds__(NT, MINB) sweep_fixed_r_kernel(SweepArgs a)
{
    using Sh = Shape<LH, HH>;
    constexpr int QPT = (Sh::CS + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lat0 = a.lat0 + (int)blockIdx.x * R;
    const int conf = lat0 / a.nrep;
    Real* Ps = reinterpret_cast<Real*>(smem + R * Sh::NB);
#pragma unroll
    for (int r = 0; r < R; ++r)
        block_copy16(smem + r * Sh::NB, a.spins + (long long)(lat0 + r) * a.lat_stride, Sh::NB);
    block_copy16_ldg(Ps, field_base<Real>(a, conf),
                     (int)((Sh::N * sizeof(Real) + 15) & ~(size_t)15));
    OffsetCache<QPT> off;
    fill_offsets<LH, HH, NT, QPT>(off, (int)threadIdx.x);
    __syncthreads();
    uint32_t* S32[R];
    int rep[R];
    double beta[R];
    float kb[R];
    Acc acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        S32[r] = reinterpret_cast<uint32_t*>(smem + r * Sh::NB);
        rep[r] = lat0 + r - conf * a.nrep;
        beta[r] = a.use_override ? a.beta_override
                                 : a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep[r]]];
        kb[r] = (float)(-2.0 * beta[r] * 1.4426950408889634);
        acc[r] = Acc{0, 0, 0, 0, 0};
    }
    const uint32_t sweep0 =
        a.use_override ? a.sweep_override : a.ctl[0] * (uint32_t)a.ptswapever;
    const uint32_t kconf = (uint32_t)conf;
#pragma unroll 1
    for (int t = 0; t < a.nsweeps; ++t)
        all_colours_r<Real, LH, HH, NT, QPT, R, false, VAC>(a, S32, Ps, off, sweep0 + (uint32_t)t,
                                                             rep, kconf, beta, kb, acc);
    all_colours_r<Real, LH, HH, NT, QPT, R, true, VAC>(a, S32, Ps, off, 0u, rep, kconf, beta, kb,
                                                        acc);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const Acc tot = block_reduce(acc[r]);
        if (threadIdx.x == 0) store_obs(a.obs + lat0 + r, tot);
        __syncthreads();  // block_reduce's scratch is reused by the next replica
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
        block_copy16(a.spins + (long long)(lat0 + r) * a.lat_stride, smem + r * Sh::NB, Sh::NB);
}

// Streaming form of the same kernel: one resident CTA per SM (MINB per SM) works through a
// contiguous range of the group's lattices.  The next lattice's spins arrive by a bulk copy of
// the tensor memory accelerator (completed on an mbarrier) into the second of two shared-memory
// buffers while the current one is swept, each finished lattice leaves by a bulk store, and the
// field stays resident while consecutive lattices are replicas of one configuration (a
// configuration's replicas are contiguous), so a CTA loads it once or twice instead of once per
// lattice.  Sweeps and results are those of sweep_fixed_kernel, bit for bit.  The two buffers
// take turns in an unrolled pair of lattice steps, so every shared-memory address of the sweeps
// stays a register offset plus an immediate.
template <class Real, int LH, int HH>
struct StreamLayout {
    using Sh = Shape<LH, HH>;
    static constexpr uint32_t SB = (uint32_t)Sh::NB;                                     // spins
    static constexpr uint32_t PB = (uint32_t)((Sh::N * sizeof(Real) + 15) & ~(size_t)15);  // field
    static constexpr uint32_t kChunk = 16384;  // bytes per bulk copy instruction
};

// Bookkeeping of the bulk loads, kept in shared memory and touched by thread 0 only (the other
// threads carry no copy of it in registers, where the sweeps need every one)
struct StreamState {
    uint32_t ph;    // bit b: parity of the phase of barrier b (spin buffer 0, 1, field) to wait for
    uint32_t pend;  // bit b: a load completing on barrier b was issued and not yet seen complete
    int field_pending;  // the field of the current configuration is still arriving
    int fail;           // a bounded wait gave up: the CTA sweeps, stores and loads nothing more
};

template <class Real, int LH, int HH>
__device__ __forceinline__ void stream_copy_in(void* dst, const void* src, uint32_t bytes,
                                               uint64_t* b)
{
    constexpr uint32_t kChunk = StreamLayout<Real, LH, HH>::kChunk;
    mbar_expect_tx(b, bytes);
    for (uint32_t o = 0; o < bytes; o += kChunk)
        bulk_load(static_cast<unsigned char*>(dst) + o, static_cast<const unsigned char*>(src) + o,
                  bytes - o < kChunk ? bytes - o : kChunk, b);
}

// One lattice of the range from spin buffer BUF (compile-time: constant shared-memory offsets).
// Thread 0 waits (bounded) for the lattice's spins and, at a configuration change, its field;
// the barrier after the wait passes the completed copies, or the failure, to every thread.  On a
// failure the CTA stops before touching the buffer: no sweep, no store and no further load.
// Returns false once stopped (the same value in every thread: read after a barrier, and written
// again only by thread 0 before the next step's barrier).
template <class Real, int LH, int HH, int NT, int QPT, bool VAC, int BUF>
__device__ __forceinline__ bool stream_step(const SweepArgs& a, unsigned char* smem, uint64_t* bar,
                                            StreamState* st, const OffsetCache<QPT>& off, int l,
                                            int last)
{
    using Lay = StreamLayout<Real, LH, HH>;
    const int tid = (int)threadIdx.x;
    Real* Ps = reinterpret_cast<Real*>(smem);
    uint32_t* S32 = reinterpret_cast<uint32_t*>(smem + Lay::PB + BUF * Lay::SB);
    const int lat = a.lat0 + l;
    if (tid == 0) {
        uint32_t ph = st->ph, pend = st->pend;
        bool ok = mbar_wait(&bar[BUF], (ph >> BUF) & 1u, a.err);
        if (ok) {
            ph ^= 1u << BUF;
            pend &= ~(1u << BUF);
            if (st->field_pending) {
                ok = mbar_wait(&bar[2], (ph >> 2) & 1u, a.err);
                if (ok) {
                    ph ^= 4u;
                    pend &= ~4u;
                    st->field_pending = 0;
                }
            }
        }
        if (ok && l + 1 < last) {  // next lattice into the other buffer
            bulk_wait_read();      // its previous lattice has left
            stream_copy_in<Real, LH, HH>(smem + Lay::PB + (BUF ^ 1) * Lay::SB,
                                         a.spins + (long long)(lat + 1) * a.lat_stride, Lay::SB,
                                         &bar[BUF ^ 1]);
            pend |= 1u << (BUF ^ 1);
        }
        st->ph = ph;
        st->pend = pend;
        if (!ok) st->fail = 1;
    }
    __syncthreads();
    if (st->fail) return false;
    const int conf = lat / a.nrep;
    const int rep = lat - conf * a.nrep;
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
    const uint32_t kconf = (uint32_t)conf;
    Acc acc{0, 0, 0, 0, 0};
#pragma unroll 1
    for (int t = 0; t < a.nsweeps; ++t)
        all_colours<Real, LH, HH, NT, QPT, false, VAC>(a, S32, Ps, off, sweep0 + (uint32_t)t,
                                                       (uint32_t)rep, kconf, beta, kb, acc);
    all_colours<Real, LH, HH, NT, QPT, true, VAC>(a, S32, Ps, off, 0u, 0u, 0u, beta, kb, acc);
    const Acc tot = block_reduce(acc);
    fence_async_shared();  // the sweeps' shared-memory accesses, before the bulk copies
    __syncthreads();
    if (tid == 0) {
        store_obs(a.obs + lat, tot);
        bulk_store(a.spins + (long long)lat * a.lat_stride, S32, Lay::SB);
        bulk_commit();
        if (l + 1 < last && (lat + 1) / a.nrep != conf) {  // the next configuration's field
            stream_copy_in<Real, LH, HH>(Ps, field_base<Real>(a, conf + 1), Lay::PB, &bar[2]);
            st->field_pending = 1;
            st->pend |= 4u;
        }
    }
    return true;
}

template <class Real, int LH, int HH, int NT, int MINB, bool VAC>
__global__ void __launch_bounds__(NT, MINB) sweep_stream_kernel(SweepArgs a, int nlat)
{
    using Sh = Shape<LH, HH>;
    using Lay = StreamLayout<Real, LH, HH>;
    constexpr int QPT = (Sh::CS + NT - 1) / NT;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar[3];  // spin buffer 0, spin buffer 1, field
    __shared__ StreamState st;
    const int tid = (int)threadIdx.x;
    const int first = (int)(((long long)blockIdx.x * nlat) / gridDim.x);
    const int last = (int)(((long long)(blockIdx.x + 1) * nlat) / gridDim.x);
    if (first >= last) return;  // uniform over the CTA: no thread waits at a barrier below
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        mbar_init_fence();
        const int lat = a.lat0 + first;
        stream_copy_in<Real, LH, HH>(smem + Lay::PB, a.spins + (long long)lat * a.lat_stride,
                                     Lay::SB, &bar[0]);
        stream_copy_in<Real, LH, HH>(smem, field_base<Real>(a, lat / a.nrep), Lay::PB, &bar[2]);
        st = StreamState{0u, 1u | 4u, 1, 0};
    }
    OffsetCache<QPT> off;
    fill_offsets<LH, HH, NT, QPT>(off, tid);
    // (the first step's barrier publishes thread 0's initialisation)
#pragma unroll 1
    for (int l = first; l < last; l += 2) {
        if (!stream_step<Real, LH, HH, NT, QPT, VAC, 0>(a, smem, bar, &st, off, l, last)) break;
        if (l + 1 < last &&
            !stream_step<Real, LH, HH, NT, QPT, VAC, 1>(a, smem, bar, &st, off, l + 1, last))
            break;
    }
    if (tid == 0) {
        // A wait gave up (err is set; the rest of the range was not swept): before the CTA's
        // shared memory is released, wait once more, again bounded, for every load that thread 0
        // issued and has not seen complete.  Outside the lattice loop, so it adds no register
        // pressure there.
        if (st.fail)
            for (int b = 0; b < 3; ++b)
                if (st.pend & (1u << b)) mbar_wait(&bar[b], (st.ph >> b) & 1u, a.err);
        bulk_wait_all();  // every stored lattice has left before the CTA ends
    }
}

template <class Real, int LH, int HH, int NT, int MINB, bool STAGE_P, bool VAC>
cudaError_t run_fixed(const SweepArgs& a, int nblocks, size_t smem, cudaStream_t st, bool prep)
{
    auto k = sweep_fixed_kernel<Real, LH, HH, NT, MINB, STAGE_P, VAC>;
    if (prep) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k<<<nblocks, NT, smem, st>>>(a);
    return cudaGetLastError();
}

// streaming form: MINB CTAs per SM (or one per lattice when there are fewer lattices)
template <class Real, int LH, int HH, int NT, int MINB, bool STAGE_P, bool VAC>
cudaError_t run_stream(const SweepArgs& a, int nlat, size_t smem, cudaStream_t st, bool prep)
{
    static_assert(STAGE_P, "the streaming form keeps the field in shared memory");
    auto k = sweep_stream_kernel<Real, LH, HH, NT, MINB, VAC>;
    if (prep) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int grid = nlat < nsm * MINB ? nlat : nsm * MINB;
    if (grid <= 0) return cudaSuccess;
    k<<<grid, NT, smem, st>>>(a, nlat);
    return cudaGetLastError();
}

// R replicas per CTA: nlat / R CTAs (whole configurations, R dividing the ladder)
template <class Real, int LH, int HH, int NT, int MINB, bool VAC, int R>
cudaError_t run_fixed_r(const SweepArgs& a, int nlat, size_t smem, cudaStream_t st, bool prep)
{
    auto k = sweep_fixed_r_kernel<Real, LH, HH, NT, MINB, VAC, R>;
    if (prep) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (a.nrep % R != 0 || a.lat0 % R != 0 || nlat % R != 0) return cudaErrorInvalidValue;
    if (nlat == 0) return cudaSuccess;
    k<<<nlat / R, NT, smem, st>>>(a);
    return cudaGetLastError();
}

using FixedFn = cudaError_t (*)(const SweepArgs&, int, size_t, cudaStream_t, bool);

struct FixedEntry {
    bool fp64;
    int L, H, nt;
    bool stage_p;
    bool vac;  // handles vacancies (entries without it are only used for vacancy-free contexts)
    FixedFn fn;
    bool stream = false;  // the streaming form
    int minb = 1;         // resident CTAs per SM the kernel is compiled for (MINB)
    int rpc = 1;          // replicas of one configuration per CTA
};

// Shapes of the reference's configurations (L = 16, 24, 32, 48 with H = L) and the CTA sizes
// the autotuner chooses from; the MINB template argument is the CTAs per SM that shared memory
// allows (it bounds the registers per thread).
const FixedEntry kFixed[] = {
    {false, 16, 16, 128, true, true, run_fixed<float, 8, 8, 128, 8, true, true>, false, 8},
    {false, 16, 16, 64, true, true, run_fixed<float, 8, 8, 64, 10, true, true>, false, 10},
    {false, 24, 24, 448, true, true, run_fixed<float, 12, 12, 448, 2, true, true>, false, 2},
    {false, 24, 24, 224, true, true, run_fixed<float, 12, 12, 224, 2, true, true>, false, 2},
    {false, 32, 32, 1024, true, false, run_fixed<float, 16, 16, 1024, 1, true, false>},
    {false, 32, 32, 512, true, false, run_fixed<float, 16, 16, 512, 1, true, false>},
    {false, 32, 32, 1024, true, true, run_fixed<float, 16, 16, 1024, 1, true, true>},
    {false, 32, 32, 512, true, true, run_fixed<float, 16, 16, 512, 1, true, true>},
    {false, 48, 48, 864, false, true, run_fixed<float, 24, 24, 864, 1, false, true>},
    {false, 48, 48, 576, false, true, run_fixed<float, 24, 24, 576, 1, false, true>},
    {true, 24, 24, 448, true, true, run_fixed<double, 12, 12, 448, 1, true, true>},
    {true, 32, 32, 512, false, true, run_fixed<double, 16, 16, 512, 1, false, true>},
    // streaming forms (the autotuner times them against the per-lattice CTAs above)
    {false, 32, 32, 1024, true, false, run_stream<float, 16, 16, 1024, 1, true, false>, true},
    {false, 32, 32, 1024, true, true, run_stream<float, 16, 16, 1024, 1, true, true>, true},
    {false, 24, 24, 448, true, true, run_stream<float, 12, 12, 448, 2, true, true>, true, 2},
    {false, 16, 16, 128, true, true, run_stream<float, 8, 8, 128, 8, true, true>, true, 8},
    // two replicas of one configuration per CTA (the autotuner times them against the above)
    {false, 32, 32, 512, true, false, run_fixed_r<float, 16, 16, 512, 1, false, 2>, false, 1, 2},
    {false, 32, 32, 512, true, true, run_fixed_r<float, 16, 16, 512, 1, true, 2>, false, 1, 2},
    {false, 24, 24, 448, true, true, run_fixed_r<float, 12, 12, 448, 2, true, 2>, false, 2, 2},
    {false, 16, 16, 128, true, true, run_fixed_r<float, 8, 8, 128, 4, true, 2>, false, 4, 2},
};

// Entries usable for a context: vacancy-free entries when it has no vacancy (where they exist),
// else the vacancy-capable ones.
bool usable(const FixedEntry& e, bool fp64, int L, int H, bool vac)
{
    if (e.fp64 != fp64 || e.L != L || e.H != H) return false;
    if (vac) return e.vac;
    for (const auto& f : kFixed)
        if (f.fp64 == fp64 && f.L == L && f.H == H && !f.vac) return !e.vac;
    return true;
}

// ---- lattices in HBM --------------------------------------------------------------------------
// Lattices too large for one CTA's shared memory (L = 96: 864 KiB of spins) keep spins and field
// in HBM / L2 and run one launch per colour phase; the kernel boundary is the barrier between
// colours.  One thread per quad with the same compile-time offsets, operand loads and arithmetic
// as the shared-memory kernel above, so the results are those of every other kernel bit for bit.
// Grid: (quads of a colour / NT, lattices).
// One colour phase of quad o in RPT replicas of one configuration: the field operands are loaded
// once and shared, the spin operands of every replica are loaded before any is updated.
template <class Real, int LH, int HH, int C, int RPT, bool VAC>
__device__ __forceinline__ void hbm_phase(const SweepArgs& a, const Real* P, const QuadOff& o,
                                          int conf, const int* rep, uint32_t sweep)
{
    QuadData<Real> d[RPT];
    load_quad_field<Real, LH, HH, C>(P, o, d[0]);
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        if (r > 0) d[r] = d[0];
        load_quad_spins<Real, LH, HH, C>(
            reinterpret_cast<const uint32_t*>(
                a.spins + (long long)(conf * a.nrep + rep[r]) * a.lat_stride),
            o, d[r]);
    }
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const double beta = a.use_override
                                ? a.beta_override
                                : a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep[r]]];
        const float kb = (float)(-2.0 * beta * 1.4426950408889634);
        Acc none{0, 0, 0, 0, 0};
        compute_quad<Real, LH, HH, C, false, VAC, true>(
            a,
            reinterpret_cast<uint32_t*>(a.spins +
                                        (long long)(conf * a.nrep + rep[r]) * a.lat_stride),
            d[r], sweep, (uint32_t)rep[r], (uint32_t)conf, beta, kb, none);
    }
}

// Grid: (quads of a colour / NT, lattices / RPT); with RPT > 1 the launcher guarantees that the
// RPT lattices of a block row are replicas of one configuration.  SLOTS: block row y covers
// temperature slots slot0 + RPT * (y % (nslots / RPT)) .. + RPT - 1 of configuration
// lat0 / nrep + y / (nslots / RPT), the lattices that hold them now (rep_at_temp).
template <class Real, int LH, int HH, int NT, int RPT, bool VAC, bool SLOTS>
__global__ void __launch_bounds__(NT, sizeof(Real) == 8 ? 1 : RPT == 4 ? 768 / NT : 1024 / NT)
    sweep_fixed_hbm_kernel(SweepArgs a, int colour, int t)
{
    pdl_wait();
    pdl_release();
    using Sh = Shape<LH, HH>;
    const int q = (int)(blockIdx.x * NT + threadIdx.x);
    if (q >= Sh::CS) return;
    int conf, rep[RPT];
    if (SLOTS) {
        const int per = a.nslots / RPT;
        conf = a.lat0 / a.nrep + (int)blockIdx.y / per;
        const int s0 = a.slot0 + ((int)blockIdx.y % per) * RPT;
#pragma unroll
        for (int r = 0; r < RPT; ++r) rep[r] = a.rep_at_temp[conf * a.nrep + s0 + r];
    } else {
        const int lat = a.lat0 + (int)blockIdx.y * RPT;
        conf = lat / a.nrep;
#pragma unroll
        for (int r = 0; r < RPT; ++r) rep[r] = lat - conf * a.nrep + r;
    }
    const Real* P = field_base<Real>(a, conf);
    const uint32_t sweep = (a.use_override ? a.sweep_override
                                           : a.ctl[0] * (uint32_t)a.ptswapever) + (uint32_t)t;
    const QuadOff o = quad_offsets<LH, HH>(q);
    switch (colour) {
#define J1J2_HBM_PHASE(C)                                                                     \
    case C:                                                                                   \
        hbm_phase<Real, LH, HH, C, RPT, VAC>(a, P, o, conf, rep, sweep);                      \
        break;
        J1J2_HBM_PHASE(0)
        J1J2_HBM_PHASE(1)
        J1J2_HBM_PHASE(2)
        J1J2_HBM_PHASE(3)
        J1J2_HBM_PHASE(4)
        J1J2_HBM_PHASE(5)
        J1J2_HBM_PHASE(6)
        J1J2_HBM_PHASE(7)
#undef J1J2_HBM_PHASE
        default:
            break;
    }
}

// Observables: one thread per quad in RPT replicas of one configuration (field operands loaded
// once), grid (quads / NT, lattices / RPT, colour); per-CTA sums are added into the lattices'
// (zeroed) observables with atomics (integer sums: order-independent).
template <class Real, int LH, int HH, int NT, int RPT, bool VAC>
__global__ void __launch_bounds__(NT) measure_fixed_hbm_kernel(SweepArgs a)
{
    pdl_wait();
    pdl_release();
    using Sh = Shape<LH, HH>;
    const int q = (int)(blockIdx.x * NT + threadIdx.x);
    const int lat = a.lat0 + (int)blockIdx.y * RPT;
    const int conf = lat / a.nrep;
    const Real* P = field_base<Real>(a, conf);
    Acc acc[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) acc[r] = Acc{0, 0, 0, 0, 0};
    if (q < Sh::CS) {
        const QuadOff o = quad_offsets<LH, HH>(q);
        switch (blockIdx.z) {
#define J1J2_HBM_MEASURE(C)                                                                     \
    case C: {                                                                                   \
        QuadData<Real> d[RPT];                                                                  \
        load_quad_field<Real, LH, HH, C>(P, o, d[0]);                                           \
        _Pragma("unroll") for (int r = 0; r < RPT; ++r)                                         \
        {                                                                                       \
            if (r > 0) d[r] = d[0];                                                             \
            load_quad_spins<Real, LH, HH, C>(                                                   \
                reinterpret_cast<const uint32_t*>(a.spins + (long long)(lat + r) * a.lat_stride), \
                o, d[r]);                                                                       \
        }                                                                                       \
        _Pragma("unroll") for (int r = 0; r < RPT; ++r)                                         \
            compute_quad<Real, LH, HH, C, true, VAC>(a, nullptr, d[r], 0u, 0u, 0u, 0.0, 0.0f,      \
                                                     acc[r]);                                   \
        break;                                                                                  \
    }
            J1J2_HBM_MEASURE(0)
            J1J2_HBM_MEASURE(1)
            J1J2_HBM_MEASURE(2)
            J1J2_HBM_MEASURE(3)
            J1J2_HBM_MEASURE(4)
            J1J2_HBM_MEASURE(5)
            J1J2_HBM_MEASURE(6)
            J1J2_HBM_MEASURE(7)
#undef J1J2_HBM_MEASURE
            default:
                break;
        }
    }
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const Acc tot = block_reduce(acc[r]);
        if (threadIdx.x == 0) {
            LatObs* ob = a.obs + lat + r;
            atomicAdd(reinterpret_cast<unsigned long long*>(&ob->eacc), (unsigned long long)tot.e);
            atomicAdd(&ob->M, tot.M);
            atomicAdd(&ob->SX, tot.SX);
            atomicAdd(&ob->SY, tot.SY);
            atomicAdd(&ob->NB, tot.NB);
        }
        __syncthreads();  // block_reduce's scratch is reused by the next replica
    }
}

template <class Real, int LH, int HH, int NT>
cudaError_t run_hbm(const SweepArgs& a, int colour, int t, int nlat, int rpt, cudaStream_t st)
{
    constexpr int CS = Shape<LH, HH>::CS;
    const unsigned gx = (unsigned)((CS + NT - 1) / NT);
    const bool pdl = a.pdl != 0;
    const dim3 b((unsigned)NT);
    if (colour < 0 && rpt == 4)
        return launch_k(pdl, dim3(gx, (unsigned)(nlat / 4), 8u), b, 0, st,
                        measure_fixed_hbm_kernel<Real, LH, HH, NT, 4, true>, a);
    if (colour < 0 && rpt == 2)
        return launch_k(pdl, dim3(gx, (unsigned)(nlat / 2), 8u), b, 0, st,
                        measure_fixed_hbm_kernel<Real, LH, HH, NT, 2, true>, a);
    if (colour < 0)
        return launch_k(pdl, dim3(gx, (unsigned)nlat, 8u), b, 0, st,
                        measure_fixed_hbm_kernel<Real, LH, HH, NT, 1, true>, a);
    if (a.nslots > 0) {  // a slot range of every configuration (nlat: whole configurations)
        const unsigned gy = (unsigned)(nlat / a.nrep * (a.nslots / rpt));
        if (rpt == 4)
            return launch_k(pdl, dim3(gx, gy), b, 0, st,
                            sweep_fixed_hbm_kernel<Real, LH, HH, NT, 4, true, true>, a, colour,
                            t);
        if (rpt == 2)
            return launch_k(pdl, dim3(gx, gy), b, 0, st,
                            sweep_fixed_hbm_kernel<Real, LH, HH, NT, 2, true, true>, a, colour,
                            t);
        return launch_k(pdl, dim3(gx, gy), b, 0, st,
                        sweep_fixed_hbm_kernel<Real, LH, HH, NT, 1, true, true>, a, colour, t);
    }
    if (rpt == 4)
        return launch_k(pdl, dim3(gx, (unsigned)(nlat / 4)), b, 0, st,
                        sweep_fixed_hbm_kernel<Real, LH, HH, NT, 4, true, false>, a, colour, t);
    if (rpt == 2)
        return launch_k(pdl, dim3(gx, (unsigned)(nlat / 2)), b, 0, st,
                        sweep_fixed_hbm_kernel<Real, LH, HH, NT, 2, true, false>, a, colour, t);
    return launch_k(pdl, dim3(gx, (unsigned)nlat), b, 0, st,
                    sweep_fixed_hbm_kernel<Real, LH, HH, NT, 1, true, false>, a, colour, t);
}

using HbmFn = cudaError_t (*)(const SweepArgs&, int, int, int, int, cudaStream_t);

struct HbmEntry {
    bool fp64;
    int L, H, nt;
    HbmFn fn;
};

// L = 96 (the reference's largest configuration) and L = 32 (a cheap cross-check of the same
// code against the shared-memory kernels); vacancy handling always on.
const HbmEntry kHbm[] = {
    {false, 96, 96, 256, run_hbm<float, 48, 48, 256>},
    {true, 96, 96, 256, run_hbm<double, 48, 48, 256>},
    {false, 32, 32, 256, run_hbm<float, 16, 16, 256>},
    {true, 32, 32, 256, run_hbm<double, 16, 16, 256>},
};

}  // namespace

int fixed_candidates(bool fp64, int L, int H, bool masks, bool vac, bool int_cpl, int nrep,
                     FixedChoice* out, int cap)
{
    if (masks || (!fp64 && !int_cpl)) return 0;
    int n = 0;
    for (const auto& e : kFixed)
        if (usable(e, fp64, L, H, vac) && nrep % e.rpc == 0 && n < cap)
            out[n++] = FixedChoice{e.nt, e.stage_p, e.stream, e.minb, e.rpc};
    return n;
}

cudaError_t launch_fixed(const SweepArgs& a, bool fp64, bool vac, const FixedChoice& ch, int nlat,
                         size_t smem, cudaStream_t st, bool prepare)
{
    for (const auto& e : kFixed)
        if (usable(e, fp64, a.g.L, a.g.H, vac) && e.nt == ch.nt && e.stream == ch.stream &&
            e.minb == ch.minb && e.rpc == ch.rpc)
            return e.fn(a, nlat, smem, st, prepare);
    return cudaErrorInvalidValue;
}

int fixed_hbm_threads(bool fp64, int L, int H, bool masks, bool int_cpl)
{
    if (masks || (!fp64 && !int_cpl)) return 0;
    for (const auto& e : kHbm)
        if (e.fp64 == fp64 && e.L == L && e.H == H) return e.nt;
    return 0;
}

cudaError_t launch_fixed_hbm(const SweepArgs& a, bool fp64, int colour, int t, int nlat, int rpt,
                             cudaStream_t st)
{
    // replicas per thread only over whole configurations (RPT lattices of one block row share
    // their configuration's field)
    if (rpt > 1 && (a.nrep % rpt != 0 || a.lat0 % a.nrep != 0 || nlat % a.nrep != 0)) rpt = 1;
    if (rpt != 2 && rpt != 4) rpt = 1;
    if (a.nslots > 0) {  // slot ranges: whole configurations, RPT dividing the range
        if (colour < 0 || a.lat0 % a.nrep != 0 || nlat % a.nrep != 0 || a.slot0 < 0 ||
            a.slot0 + a.nslots > a.nrep)
            return cudaErrorInvalidValue;
        while (rpt > 1 && a.nslots % rpt != 0) rpt /= 2;
    }
    for (const auto& e : kHbm)
        if (e.fp64 == fp64 && e.L == a.g.L && e.H == a.g.H)
            return e.fn(a, colour, t, nlat, rpt, st);
    return cudaErrorInvalidValue;
}

}  // namespace j1j2
