// Wolff cluster update for every lattice of a group (named in the reference's header comment,
// J:7, but never implemented there).  For the Ising Hamiltonian E = -sum_<ij> K_ij s_i s_j with the
// per-bond couplings of Compute_local_field (J:2498-2541) -- K = J1h*jh + p_i + p_j on x bonds,
// J1v*jv - p_i - p_j on y bonds, J2 on diagonals, J3 between layers -- a bond with K s_i s_j > 0 is
// activated with probability 1 - exp(-2 beta K s_i s_j); the connected component of a seed site
// is flipped.  The model has no field on s, so the move satisfies detailed balance for any sign of
// K.  Bonds are enumerated once from their owner site (+x, +y, (+x,+y), (-x,+y), +z); when L = 2 or
// H = 2 a pair is reached from both sides and receives two trials, i.e. coupling 2K, exactly as
// the doubled neighbour slots of the reference (J:564-574).
//
// Three forms flip the same cluster.  The default grows the seed's cluster breadth-first (one CTA
// per lattice, only the bonds of the cluster and its boundary are tested; see the growth kernel
// below).  The two labelling forms label every component and then flip the seed's; they are kept
// as cross-checks and selectable by flags.
//
// Labelling: components are labelled in a scratch array (one int32 per site, the compact index
// of a site of the same component) by lock-free union-find: hooking the larger root under the
// smaller with atomicCAS, path halving in find, so every pointer goes to a smaller compact index
// and every root is the smallest compact index of its component.  Then the seed's component is flipped.
//
// Slab form (lattices up to 65536 sites per two planes): one CTA per slab of pz planes
// (pz even, a divisor of H) stages the slab's spins in shared memory and runs the union-find on
// 16-bit slab-local indices ordered like the compact layout (colour-major, each colour's planes
// contiguous), which keeps the root of every slab-local component at its smallest compact index;
// it writes every site's global label as that root.  A second kernel unites the +z bonds that
// leave a slab in global memory, and the flip kernel finds roots on the fly.  Components, and so
// the flipped cluster, are those of the site-per-thread global form, which stays as the path for
// larger planes and for the per-site test mode.
//
// Streams (Philox4x32-10, key = (seed, conf_base + conf)):
//   in-plane bond b = 0..3 of the site with compact index i: ctr = (replica, cycle, i, 5), word b
//   +z bond of the site in group g:  ctr = (replica, cycle, g, 3 + 16*4), word X & 3
//   (one call draws a site's four in-plane words: the growth form, which tests a site's bonds
//   site by site, needs seven calls per cluster site instead of ten)
//   seed site:                     ctr = (replica, cycle, 0xFFFFFFFF, 4), word 0; the site is
//                                  floor(w * N / 2^32) in reference site order; a vacancy seed
//                                  means no flip this cycle (a configuration-independent choice)
#include <cooperative_groups.h>

#include "sweep_common.cuh"

namespace cg = cooperative_groups;

namespace j1j2 {
namespace {

enum : uint32_t { kTagWolffBond = 3u, kTagWolffSeed = 4u, kTagWolffSite = 5u };
constexpr uint32_t kTagWolffZ = kTagWolffBond + 16u * 4u;  // the +z bond's tag

struct SiteCoord {
    int x, y, z;
};

__device__ __forceinline__ SiteCoord coord_of_compact(const Geo& g, int ci)
{
    const int c = ci / g.Nc, k = ci - c * g.Nc;
    const int X = k % g.Lh, r = k / g.Lh;
    const int Y = r % g.Lh, Z = r / g.Lh;
    return SiteCoord{2 * X + (c & 1), 2 * Y + ((c >> 1) & 1), 2 * Z + (c >> 2)};
}

__device__ __forceinline__ int compact_of_xyz(const Geo& g, int x, int y, int z)
{
    const int c = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
    return cidx(g, c, z >> 1, y >> 1, x >> 1);
}

// find with path halving; labels are read through volatile loads (other threads hook roots)
__device__ __forceinline__ int find_root(volatile int* lab, int x)
{
    int p = lab[x];
    while (p != x) {
        const int gp = lab[p];
        if (gp != p) lab[x] = gp;  // only ever moves a pointer closer to its root
        x = p;
        p = gp;
    }
    return x;
}

// Union of the components of a and b; false if the retry budget (tries attempts, SweepArgs::
// uf_tries) ran out (the caller sets the error word).
__device__ __forceinline__ bool unite(volatile int* lab, int a, int b, int tries)
{
    for (int it = 0; it < tries; ++it) {
        a = find_root(lab, a);
        b = find_root(lab, b);
        if (a == b) return true;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        // hook the larger root a under b; fails if a stopped being a root meanwhile
        if (atomicCAS(const_cast<int*>(lab) + a, a, b) == a) return true;
    }
    return false;
}

template <class Real>
__device__ __forceinline__ const Real* wfield(const SweepArgs& a, int conf)
{
    if constexpr (sizeof(Real) == 8)
        return a.pd + (long long)conf * a.p_stride;
    else
        return a.pf + (long long)conf * a.p_stride;
}

// Weight w = K_ij s_i s_j of the bond of type b (coupling K_ij as in Compute_local_field); true
// if the bond can be activated (w > 0).
template <class Real>
__device__ __forceinline__ bool bond_weight(const SweepArgs& a, int b, int si, int sj, int jh,
                                            int jv, Real pi, Real pj, Real& w)
{
    Real K;
    if constexpr (sizeof(Real) == 8) {
        if (b == 0)
            K = __dadd_rn(__dadd_rn(jh ? a.J1h : 0.0, pi), pj);
        else if (b == 1)
            K = __dsub_rn(__dsub_rn(jv ? a.J1v : 0.0, pi), pj);
        else if (b < 4)
            K = a.J2;
        else
            K = a.J3;
    } else {
        if (b == 0)
            K = __fadd_rn(__fadd_rn(jh ? a.J1hf : 0.0f, pi), pj);
        else if (b == 1)
            K = __fsub_rn(__fsub_rn(jv ? a.J1vf : 0.0f, pi), pj);
        else if (b < 4)
            K = a.J2f;
        else
            K = a.J3f;
    }
    w = si * sj > 0 ? K : -K;
    return w > Real(0);
}

// The FP32 trials' scale (float)(-2 beta log2(e)), computed once per lattice: two FP64
// multiplies and a conversion, which GB300 runs at ~64 clocks each, kept out of the per-bond path
__device__ __forceinline__ float trial_scale(double beta)
{
    return (float)(-2.0 * beta * 1.4426950408889634);
}

// Activation trial of a bond of weight w > 0 with the uniform of word r: u < 1 - exp(-2 beta w)
// (FP32: kb = trial_scale(beta))
template <class Real>
__device__ __forceinline__ bool bond_trial(Real w, double beta, float kb, uint32_t r)
{
    if constexpr (sizeof(Real) == 8) {
        const double pa = __dsub_rn(1.0, own_exp(-__dmul_rn(__dmul_rn(2.0, w), beta)));
        return u01_f64(r) < pa;
    } else {
        const float pa = __fsub_rn(1.0f, ex2_approx(__fmul_rn(kb, w)));
        return u01_f32(r) < pa;
    }
}

__global__ void wolff_init_kernel(int* labels, long long lab_stride, int N)
{
    int* lab = labels + (long long)blockIdx.y * lab_stride;
    for (int i = (int)(blockIdx.x * blockDim.x + threadIdx.x); i < N;
         i += (int)(gridDim.x * blockDim.x))
        lab[i] = i;
}

template <class Real, bool MASKS>
__global__ void __launch_bounds__(256) wolff_bond_kernel(SweepArgs a, int* labels,
                                                         long long lab_stride, int* err)
{
    const Geo g = a.g;
    const int lat = (int)blockIdx.y;
    const int conf = lat / a.nrep, rep = lat - conf * a.nrep;
    const int ci = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (ci >= g.N) return;
    const uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    const int si = (int)S[ci] - 1;
    if (si == 0) return;
    const Real* P = wfield<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    volatile int* lab = labels + (long long)lat * lab_stride;
    const double beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
    const float kbw = trial_scale(beta);
    const uint32_t cycle = a.ctl[0];
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    const SiteCoord s = coord_of_compact(g, ci);
    const int c = ci / g.Nc;
    const int X = s.x >> 1;
    const uint32_t grp =
        (uint32_t)(((c * g.Hh + (s.z >> 1)) * g.Lh + (s.y >> 1)) * g.Qr + (X >> 2));
    const int xp = s.x + 1 == g.L ? 0 : s.x + 1, xm = s.x == 0 ? g.L - 1 : s.x - 1;
    const int yp = s.y + 1 == g.L ? 0 : s.y + 1, zp = s.z + 1 == g.H ? 0 : s.z + 1;
    const int nb[5] = {compact_of_xyz(g, xp, s.y, s.z), compact_of_xyz(g, s.x, yp, s.z),
                       compact_of_xyz(g, xp, yp, s.z), compact_of_xyz(g, xm, yp, s.z),
                       compact_of_xyz(g, s.x, s.y, zp)};
    const int jh = MASKS ? (BM[ci] & 1) : 1, jv = MASKS ? ((BM[ci] >> 1) & 1) : 1;
    const Real pi = P[ci];
    const U4 inplane = philox4x32_10((uint32_t)rep, cycle, (uint32_t)ci, kTagWolffSite, k0, k1);
#pragma unroll
    for (int b = 0; b < 5; ++b) {
        const int cj = nb[b];
        const int sj = (int)S[cj] - 1;
        if (sj == 0) continue;
        Real w;
        if (!bond_weight<Real>(a, b, si, sj, jh, jv, pi, b < 2 ? P[cj] : Real(0), w)) continue;
        const uint32_t r =
            b < 4 ? u4_word(inplane, b)
                  : u4_word(philox4x32_10((uint32_t)rep, cycle, grp, kTagWolffZ, k0, k1), X & 3);
        if (bond_trial<Real>(w, beta, kbw, r) && !unite(lab, ci, cj, a.uf_tries))
            atomicExch(err, 1);
    }
}

// ---- slab form -------------------------------------------------------------------------------
__device__ __forceinline__ int sfind(volatile uint16_t* lab, int x)
{
    int p = lab[x];
    while (p != x) {
        const int gp = lab[p];
        if (gp != p) lab[x] = (uint16_t)gp;
        x = p;
        p = gp;
    }
    return x;
}

// Slab geometry: pz planes starting at plane z0 = slab * pz (pz even); the slab holds Zh = pz/2
// compact planes of each colour, local index ((c * Zh + Zl) * Lh + Y) * Lh + X.
struct Slab {
    int Zh, chunk, z0h;  // compact planes per colour, sites per colour chunk, first compact plane
    bool wrap;           // the slab is the whole lattice (+z of its last plane stays inside)
};

// x / d for 0 <= x < 2^16, 1 <= d <= 2^16 by a multiply-high with m = floor((2^32 - 1) / d) + 1:
// m*d - 2^32 < d and x*d < 2^32 keep the quotient exact.
struct FastDiv {
    uint32_t d, m;
    __device__ explicit FastDiv(uint32_t dv) : d(dv), m(dv == 1u ? 0u : 0xFFFFFFFFu / dv + 1u) {}
    __device__ __forceinline__ uint32_t operator()(uint32_t x) const
    {
        return d == 1u ? x : __umulhi(x, m);
    }
};

// Slab-local index of the neighbour of bond b of the site (c, Zl, Y, X) (bond b never leaves
// the slab here: +z bonds out of a slab that is not the whole lattice are the boundary kernel's)
__device__ __forceinline__ int slab_nbr(const Geo& g, const Slab& sl, int c, int Zl, int Y, int X,
                                        int b)
{
    const int px = c & 1, py = (c >> 1) & 1, pzb = c >> 2;
    int Zn = Zl, Yn = Y, Xn = X;
    if (b == 0 || b == 2) Xn = px ? (X + 1 == g.Lh ? 0 : X + 1) : X;   // x + 1
    if (b == 3) Xn = px ? X : (X == 0 ? g.Lh - 1 : X - 1);             // x - 1
    if (b >= 1 && b <= 3) Yn = py ? (Y + 1 == g.Lh ? 0 : Y + 1) : Y;   // y + 1
    if (b == 4) {
        Zn = Zl + pzb;
        if (Zn == sl.Zh) Zn = 0;
    }
    const int cn = c ^ (b == 0 ? 1 : b == 1 ? 2 : b < 4 ? 3 : 4);
    return ((cn * sl.Zh + Zn) * g.Lh + Yn) * g.Lh + Xn;
}

// Exact integer form of the activation trial u < pa for a bond of uniform coupling: the
// uniform's integer numerator (FP32: r mod 2^23 over 2^23; FP64: rotl(r, 9) over 2^32) is
// below ceil(pa * 2^23) (resp. 2^32), pa * 2^k being exact.
template <class Real>
__device__ __forceinline__ unsigned long long uniform_threshold(Real K, double beta)
{
    if (!(K > Real(0))) return 0ull;
    if constexpr (sizeof(Real) == 8) {
        const double pa = __dsub_rn(1.0, own_exp(-__dmul_rn(__dmul_rn(2.0, K), beta)));
        return (unsigned long long)ceil(__dmul_rn(pa, 4294967296.0));
    } else {
        const float pa = __fsub_rn(1.0f, ex2_approx(__fmul_rn(trial_scale(beta), K)));
        return (unsigned long long)ceilf(__fmul_rn(pa, 8388608.0f));
    }
}

template <class Real>
__device__ __forceinline__ bool uniform_trial(unsigned long long thr, uint32_t r)
{
    if constexpr (sizeof(Real) == 8)
        return (unsigned long long)((r << 9) | (r >> 23)) < thr;
    else
        return (unsigned long long)(r & 0x007FFFFFu) < thr;
}

// Union-find of one slab of one lattice in shared memory; writes the label of every site.
// Phase A evaluates the five owned bonds of every quad (the four sites of one Philox block) and
// keeps the activated ones in bits 2..6 of each site's staged byte (bits 0..1 keep the biased
// spin).  Phase B unites along them as a warp-synchronous state machine: in every round each lane
// takes one step (fetch a bond, one find step with path halving, or one hook attempt), so lanes
// never replay the union code for small subsets as nested divergent loops would.  Phase C writes
// every site's label, the compact index of its slab-local root.
template <class Real, bool MASKS>
__global__ void __launch_bounds__(512, 2)
    wolff_slab_kernel(SweepArgs a, int pz, int* labels, long long lab_stride, int* err)
{
    extern __shared__ __align__(16) unsigned char wsm[];
    const Geo g = a.g;
    const int lat = (int)blockIdx.y;
    const int conf = lat / a.nrep, rep = lat - conf * a.nrep;
    Slab sl;
    sl.Zh = pz >> 1;
    sl.chunk = sl.Zh * g.Lh * g.Lh;
    sl.z0h = (int)blockIdx.x * sl.Zh;
    sl.wrap = pz == g.H;
    const int nsite = 8 * sl.chunk;
    volatile uint16_t* slab = reinterpret_cast<uint16_t*>(wsm);
    uint8_t* ss = wsm + 2 * (size_t)nsite;
    const uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    const Real* P = wfield<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    int* lab = labels + (long long)lat * lab_stride;
    const int dc = g.Nc - sl.chunk, goff = sl.z0h * g.Lh * g.Lh;  // local li -> c*dc + goff + li
    const int NT = (int)blockDim.x;
    for (int c = 0; c < 8; ++c) {
        const uint8_t* src = S + c * g.Nc + goff;
        for (int k = (int)threadIdx.x; k < sl.chunk; k += NT) {
            ss[c * sl.chunk + k] = src[k];
            slab[c * sl.chunk + k] = (uint16_t)(c * sl.chunk + k);
        }
    }
    __syncthreads();

    // ---- phase A: activated bonds --------------------------------------------------------
    const double beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
    const float kbw = trial_scale(beta);
    const uint32_t cycle = a.ctl[0];
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    Real J2, J3;
    if constexpr (sizeof(Real) == 8) {
        J2 = a.J2;
        J3 = a.J3;
    } else {
        J2 = a.J2f;
        J3 = a.J3f;
    }
    const unsigned long long thr2 = uniform_threshold<Real>(J2 < Real(0) ? -J2 : J2, beta);
    const unsigned long long thr3 = uniform_threshold<Real>(J3 < Real(0) ? -J3 : J3, beta);
    const int s2 = J2 > Real(0) ? 1 : J2 < Real(0) ? -1 : 0;  // s_i s_j of a satisfied bond
    const int s3 = J3 > Real(0) ? 1 : J3 < Real(0) ? -1 : 0;
    const int rowq = g.Lh * g.Qr;
    const int cq = sl.Zh * rowq;
    const int nquad = 8 * cq;
    const FastDiv div_cq((uint32_t)cq), div_rq((uint32_t)rowq), div_qr((uint32_t)g.Qr);
    for (int q = (int)threadIdx.x; q < nquad; q += NT) {
        const int c = (int)div_cq((uint32_t)q);
        int r = q - c * cq;
        const int Zl = (int)div_rq((uint32_t)r);
        r -= Zl * rowq;
        const int Y = (int)div_qr((uint32_t)r), Xq = r - Y * g.Qr;
        const int X0 = 4 * Xq;
        const int nw = g.Lh - X0 < 4 ? g.Lh - X0 : 4;
        const int row0 = ((c * sl.Zh + Zl) * g.Lh + Y) * g.Lh;
        const bool zleave = (c >> 2) && Zl + 1 == sl.Zh && !sl.wrap;  // boundary kernel's bond
        const uint32_t grp = (uint32_t)(((c * g.Hh + sl.z0h + Zl) * g.Lh + Y) * g.Qr + Xq);
        int si[4];
#pragma unroll
        for (int w = 0; w < 4; ++w) si[w] = w < nw ? (int)(ss[row0 + X0 + w] & 3u) - 1 : 0;
        unsigned act = 0;  // bit 5*w + b
        U4 srr[4];         // each site's in-plane words, drawn when first needed
        unsigned have = 0;
#pragma unroll
        for (int b = 0; b < 5; ++b) {
            if (b == 4 && zleave) break;
            unsigned want = 0;
            Real wv[4];
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                wv[w] = Real(0);
                if (si[w] == 0) continue;
                const int lj = slab_nbr(g, sl, c, Zl, Y, X0 + w, b);
                const int ssj = si[w] * ((int)(ss[lj] & 3u) - 1);
                if (ssj == 0) continue;
                if (b < 2) {
                    const int gi = c * dc + goff + row0 + X0 + w;
                    int jh = 1, jv = 1;
                    if (MASKS) {
                        jh = BM[gi] & 1;
                        jv = (BM[gi] >> 1) & 1;
                    }
                    if (bond_weight<Real>(a, b, ssj, 1, jh, jv, P[gi],
                                          P[(c ^ (b + 1)) * dc + goff + lj], wv[w]))
                        want |= 1u << w;
                } else if (ssj == (b < 4 ? s2 : s3)) {
                    want |= 1u << w;
                }
            }
            if (!want) continue;
            U4 rr{0, 0, 0, 0};
            if (b == 4) rr = philox4x32_10((uint32_t)rep, cycle, grp, kTagWolffZ, k0, k1);
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                if (!((want >> w) & 1u)) continue;
                // in-plane bonds: word b of the site's own call
                if (b < 4 && !((have >> w) & 1u)) {
                    srr[w] = philox4x32_10((uint32_t)rep, cycle,
                                           (uint32_t)(c * dc + goff + row0 + X0 + w),
                                           kTagWolffSite, k0, k1);
                    have |= 1u << w;
                }
                const uint32_t word = b == 4 ? u4_word(rr, w) : u4_word(srr[w], b);
                const bool on = b < 2 ? bond_trial<Real>(wv[w], beta, kbw, word)
                                      : uniform_trial<Real>(b < 4 ? thr2 : thr3, word);
                if (on) act |= 1u << (5 * w + b);
            }
        }
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const unsigned m = (act >> (5 * w)) & 31u;
            if (m) ss[row0 + X0 + w] = (uint8_t)(ss[row0 + X0 + w] | (m << 2));
        }
    }
    __syncthreads();

    // ---- phase B: unions, one step per lane per round -------------------------------------
    {
        enum { kFetch = 0, kFindA = 1, kFindB = 2, kHook = 3 };
        const FastDiv div_chunk((uint32_t)sl.chunk), div_plane((uint32_t)(g.Lh * g.Lh)),
            div_lh((uint32_t)g.Lh);
        int li = (int)threadIdx.x - NT;  // site whose bonds are being united
        unsigned m = 0;                  // its bonds still to unite
        int c = 0, Zl = 0, Y = 0, X = 0;
        int st = kFetch, ua = 0, ub = 0, x = 0, tries = 0;
        bool alive = true, ok = true;
        while (__any_sync(0xFFFFFFFFu, alive)) {
            if (!alive) continue;
            if (st == kFetch) {
                if (m == 0) {
                    li += NT;
                    if (li >= nsite) {
                        alive = false;
                        continue;
                    }
                    m = (unsigned)ss[li] >> 2;
                    c = (int)div_chunk((uint32_t)li);
                    int r = li - c * sl.chunk;
                    Zl = (int)div_plane((uint32_t)r);
                    r -= Zl * g.Lh * g.Lh;
                    Y = (int)div_lh((uint32_t)r);
                    X = r - Y * g.Lh;
                } else {
                    const int b = __ffs((int)m) - 1;
                    m &= m - 1;
                    ua = li;
                    ub = slab_nbr(g, sl, c, Zl, Y, X, b);
                    x = ua;
                    st = kFindA;
                    tries = 0;
                }
            } else if (st != kHook) {  // one find step with path halving
                const int p = slab[x];
                if (p == x) {
                    if (st == kFindA) {
                        ua = x;
                        x = ub;
                        st = kFindB;
                    } else {
                        ub = x;
                        st = kHook;
                    }
                } else {
                    const int gp = slab[p];
                    if (gp != p) slab[x] = (uint16_t)gp;
                    x = p;
                }
            } else {  // hook the larger root under the smaller
                if (ua == ub) {
                    st = kFetch;
                } else {
                    const int hi = ua > ub ? ua : ub, lo = ua ^ ub ^ hi;
                    const unsigned short old = atomicCAS(
                        const_cast<unsigned short*>(reinterpret_cast<volatile unsigned short*>(slab)) + hi,
                        (unsigned short)hi, (unsigned short)lo);
                    if (old == (unsigned short)hi) {
                        st = kFetch;
                    } else if (++tries >= a.uf_tries) {  // retry budget spent: give up this bond
                        ok = false;
                        st = kFetch;
                    } else {  // hi stopped being a root: find both roots again
                        ua = hi;
                        ub = lo;
                        x = ua;
                        st = kFindA;
                    }
                }
            }
        }
        if (!ok) atomicExch(err, 1);
    }
    __syncthreads();

    // ---- phase C: labels -----------------------------------------------------------------
    const FastDiv div_chunk((uint32_t)sl.chunk);
    for (int c = 0; c < 8; ++c)
        for (int k = (int)threadIdx.x; k < sl.chunk; k += NT) {
            const int root = sfind(slab, c * sl.chunk + k);
            lab[c * g.Nc + goff + k] = (int)div_chunk((uint32_t)root) * dc + goff + root;
        }
}

// +z bonds from the last plane of every slab into the next slab (pz < H), united in global memory
template <class Real>
__global__ void __launch_bounds__(256) wolff_boundary_kernel(SweepArgs a, int pz, int* labels,
                                                             long long lab_stride, int* err)
{
    const Geo g = a.g;
    const int lat = (int)blockIdx.y;
    const int conf = lat / a.nrep, rep = lat - conf * a.nrep;
    const int nslab = g.H / pz;
    const int per_slab = 4 * g.Lh * g.Qr;  // quads of the colours of odd z in one plane
    const int item = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (item >= nslab * per_slab) return;
    const int slab = item / per_slab;
    int r = item - slab * per_slab;
    const int c = 4 + r / (g.Lh * g.Qr);
    r -= (c - 4) * g.Lh * g.Qr;
    const int Y = r / g.Qr, Xq = r - Y * g.Qr;
    const int Z = slab * (pz >> 1) + (pz >> 1) - 1;  // compact plane of z = z0 + pz - 1 (odd)
    const int Zn = Z + 1 == g.Hh ? 0 : Z + 1;
    const uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    volatile int* lab = labels + (long long)lat * lab_stride;
    const double beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
    const float kbw = trial_scale(beta);
    const uint32_t grp = (uint32_t)(((c * g.Hh + Z) * g.Lh + Y) * g.Qr + Xq);
    const U4 rr = philox4x32_10((uint32_t)rep, a.ctl[0], grp, kTagWolffZ, a.seed,
                                a.conf_base + (uint32_t)conf);
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const int X = 4 * Xq + w;
        if (X >= g.Lh) break;
        const int ci = cidx(g, c, Z, Y, X), cj = cidx(g, c ^ 4, Zn, Y, X);
        const int si = (int)S[ci] - 1, sj = (int)S[cj] - 1;
        if (si == 0 || sj == 0) continue;
        Real wv;
        if (!bond_weight<Real>(a, 4, si, sj, 1, 1, Real(0), Real(0), wv)) continue;
        if (bond_trial<Real>(wv, beta, kbw, u4_word(rr, w)) && !unite(lab, ci, cj, a.uf_tries))
            atomicExch(err, 1);
    }
}

// Flip the component of the seed site (roots found on the fly; labels of either form)
__global__ void wolff_flip_kernel(SweepArgs a, int* labels, long long lab_stride,
                                  long long* csize)
{
    const Geo g = a.g;
    const int lat = (int)blockIdx.y;
    const int conf = lat / a.nrep, rep = lat - conf * a.nrep;
    uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    volatile int* lab = labels + (long long)lat * lab_stride;
    const uint32_t w = philox4x32_10((uint32_t)rep, a.ctl[0], 0xFFFFFFFFu, kTagWolffSeed, a.seed,
                                     a.conf_base + (uint32_t)conf).x;
    const int seed_site = (int)(((unsigned long long)w * (unsigned long long)g.N) >> 32);
    const int cs = compact_of_site(g, seed_site);
    int count = 0;
    if (S[cs] != 1) {
        const int root = find_root(lab, cs);
        for (int i = (int)(blockIdx.x * blockDim.x + threadIdx.x); i < g.N;
             i += (int)(gridDim.x * blockDim.x))
            if (find_root(lab, i) == root) {
                S[i] = (uint8_t)(2 - S[i]);
                ++count;
            }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) count += __shfl_down_sync(0xFFFFFFFFu, count, o);
    if ((threadIdx.x & 31) == 0 && count) atomicAdd((unsigned long long*)(csize + lat), count);
}

// ---- seed-cluster growth ----------------------------------------------------------------------
// One CTA per lattice grows the seed's cluster breadth-first.  A bond is tested when the growth
// first reaches it, with the same owner-site Philox word, coupling and arithmetic as the
// labelling forms, so the flipped cluster is the same component; only the bonds of the cluster
// and of its boundary are evaluated.  A site joins by setting bit 2 of its spin byte with an
// atomic OR on the word holding it: the old word tells whether it had already joined and gives
// its original spin, so one round trip both claims and reads it.  The winner flips the spin
// (atomic XOR of bit 1) and appends (compact coordinates c:3 Z:9 Y:9 X:9 bits, original byte:
// 2 bits) to the cluster list; level k of the
// breadth-first search is the list segment appended during level k - 1, kept in a shared-memory
// ring while it fits.  A test that reads a neighbour already claimed by a concurrent winner sees
// bit 2 (or loses the claim), so nothing changes.  The join bits are cleared at the end.
constexpr int kGrowThreads = 1024;
constexpr int kGrowRing = 8192;  // queue entries kept in shared memory (32 KiB)
// An empty list entry: every entry has a Z below 256 (H <= 512), so its bits 28..20 are never all
// set.  The growth list is all empty entries between updates (allocation fills it, every growth
// empties what it wrote), which the level-free growth needs to see an entry arrive.
constexpr int kGrowEmpty = -1;

// CS > 1: a thread-block cluster of CS CTAs grows one lattice's cluster (levels of thousands of
// sites in the coldest lattices are bound by one SM's issue rate).  The frontier ring and the
// counters live in the shared memory of the cluster's first CTA; every CTA takes a share of a
// level's sites, appends through that CTA's counter (a distributed-shared-memory atomic) and
// meets the others at a cluster barrier between levels, whose release / acquire ordering makes
// the level's appends (ring, cluster list) visible to all.
enum : int { kCtlHead = 0, kCtlEnd = 1, kCtlTail = 2, kCtlRlim = 3, kCtlWlim = 4 };

// One cluster site of the growth: entry e (compact coordinates, original spin byte) tests its ten
// bonds and claims every neighbour an activated bond reaches; append(entry) queues each new
// cluster site.  Shared by the level-synchronous and the level-free growth kernels.
struct GrowLattice {
    uint8_t* S;        // the lattice's spin bytes
    uint32_t* S32;     // the same as words (claims and flips are word atomics)
    const uint8_t* A;  // BITS: the activation bytes of the lattice
    int rep;
    uint32_t cycle, k0, k1;
    double beta;
    float kb;                       // trial_scale(beta)
    unsigned long long thr2, thr3;  // uniform thresholds of the J2 and J3 bonds
    int s2, s3;                     // s_i s_j of a satisfied J2 / J3 bond
};

template <class Real, bool MASKS, bool BITS, class Append>
__device__ __forceinline__ void grow_entry(const SweepArgs& a, const Geo& g, const Real* P,
                                           const uint8_t* BM, const GrowLattice& w, uint32_t e,
                                           Append& append)
{
    uint8_t* S = w.S;
    uint32_t* S32 = w.S32;
    const int rep = w.rep;
    const uint32_t cycle = w.cycle, k0 = w.k0, k1 = w.k1;
    const double beta = w.beta;
    const float kbw = w.kb;
    const unsigned long long thr2 = w.thr2, thr3 = w.thr3;
    const int s2 = w.s2, s3 = w.s3;
        const int c = (int)(e >> 29), Z = (int)((e >> 20) & 511), Y = (int)((e >> 11) & 511),
                  X = (int)((e >> 2) & 511);
        const int si = (int)(e & 3u) - 1;  // original spin
        const int i = cidx(g, c, Z, Y, X);
        const int px = c & 1, py = (c >> 1) & 1, pz = c >> 2;
        const int Xp = px ? (X + 1 == g.Lh ? 0 : X + 1) : X;   // column of x + 1
        const int Xm = px ? X : (X == 0 ? g.Lh - 1 : X - 1);   // column of x - 1
        const int Yp = py ? (Y + 1 == g.Lh ? 0 : Y + 1) : Y;
        const int Ym = py ? Y : (Y == 0 ? g.Lh - 1 : Y - 1);
        const int Zp = pz ? (Z + 1 == g.Hh ? 0 : Z + 1) : Z;
        const int Zm = pz ? Z : (Z == 0 ? g.Hh - 1 : Z - 1);
        // neighbour d: +x, +y, (+x,+y), (-x,+y), +z own the bond (b = d); -x, -y, (-x,-y),
        // (+x,-y), -z are the bonds b = d - 5 owned by the neighbour
        auto cof = [&](int d) {
            return c ^ (d % 5 == 0 ? 1 : d % 5 == 1 ? 2 : d % 5 == 4 ? 4 : 3);
        };
        auto xof = [&](int d) {
            return (d == 0 || d == 2 || d == 8) ? Xp : (d == 3 || d == 5 || d == 7) ? Xm : X;
        };
        auto yof = [&](int d) {
            return (d == 1 || d == 2 || d == 3) ? Yp : (d == 6 || d == 7 || d == 8) ? Ym : Y;
        };
        auto zof = [&](int d) { return d == 4 ? Zp : d == 9 ? Zm : Z; };
        int jn[10], bn[10];
#pragma unroll
        for (int d = 0; d < 10; ++d) jn[d] = cidx(g, cof(d), zof(d), yof(d), xof(d));
        // every load first (independent, in flight together)
#pragma unroll
        for (int d = 0; d < 10; ++d) bn[d] = S[jn[d]];
        unsigned act_bits = 0;
        if constexpr (BITS) {
            // own bonds from the site's byte, the others from their owners' bytes
            const uint8_t* A = w.A;
            unsigned ab = A[i] & 31u;
#pragma unroll
            for (int d = 5; d < 10; ++d) ab |= (((unsigned)A[jn[d]] >> (d - 5)) & 1u) << d;
#pragma unroll
            for (int d = 0; d < 10; ++d) {
                const int sj = (bn[d] & 3) - 1;
                if (sj == 0 || (bn[d] & 4)) continue;  // vacancy, or joined already
                if ((ab >> d) & 1u) act_bits |= 1u << d;
            }
        } else {
            const Real p_i = P[i], p0 = P[jn[0]], p1 = P[jn[1]], p5 = P[jn[5]],
                       p6 = P[jn[6]];
            int m_i = 3, m5 = 3, m6 = 3;
            if (MASKS) {
                m_i = BM[i];
                m5 = BM[jn[5]];
                m6 = BM[jn[6]];
            }
            // the bonds' Philox words as independent chains while the loads are in flight:
            // the site's own in-plane call (bonds 0-3), its +z call, each in-plane
            // neighbour's own call (the word of the bond it owns) and the -z neighbour's +z
            // call
            uint32_t word[10];
            {
                const U4 own = philox4x32_10((uint32_t)rep, cycle, (uint32_t)i,
                                             kTagWolffSite, k0, k1);
                word[0] = own.x;
                word[1] = own.y;
                word[2] = own.z;
                word[3] = own.w;
            }
#pragma unroll
            for (int d = 4; d < 10; ++d) {
                const int b = d < 5 ? d : d - 5;
                if (b < 4) {
                    word[d] = u4_word(philox4x32_10((uint32_t)rep, cycle, (uint32_t)jn[d],
                                                    kTagWolffSite, k0, k1),
                                      b);
                } else {
                    const int co = d < 5 ? c : cof(d), Zo = d < 5 ? Z : zof(d);
                    const int Yo = d < 5 ? Y : yof(d), Xo = d < 5 ? X : xof(d);
                    const uint32_t grp =
                        (uint32_t)(((co * g.Hh + Zo) * g.Lh + Yo) * g.Qr + (Xo >> 2));
                    word[d] = u4_word(
                        philox4x32_10((uint32_t)rep, cycle, grp, kTagWolffZ, k0, k1), Xo & 3);
                }
            }
#pragma unroll
            for (int d = 0; d < 10; ++d) {
                const int sj = (bn[d] & 3) - 1;
                if (sj == 0 || (bn[d] & 4)) continue;  // vacancy, or joined already
                const int b = d < 5 ? d : d - 5;
                bool on;
                if (b < 2) {
                    const int mo = d < 5 ? m_i : (d == 5 ? m5 : m6);
                    const Real po = d < 5 ? p_i : (d == 5 ? p5 : p6);
                    const Real pt = d == 0 ? p0 : d == 1 ? p1 : p_i;
                    Real wv;
                    on = bond_weight<Real>(a, b, si, sj, mo & 1, (mo >> 1) & 1, po, pt,
                                           wv) &&
                         bond_trial<Real>(wv, beta, kbw, word[d]);
                } else {
                    on = si * sj == (b < 4 ? s2 : s3) &&
                         uniform_trial<Real>(b < 4 ? thr2 : thr3, word[d]);
                }
                if (on) act_bits |= 1u << d;
            }
        }
        // claims: every atomic issued before any result is used
        uint32_t old[10];
#pragma unroll
        for (int d = 0; d < 10; ++d)
            old[d] = ((act_bits >> d) & 1u)
                         ? atomicOr(&S32[jn[d] >> 2], 4u << (8 * (jn[d] & 3)))
                         : 4u << (8 * (jn[d] & 3));
#pragma unroll
        for (int d = 0; d < 10; ++d) {
            const int sh = 8 * (jn[d] & 3);
            if ((old[d] >> sh) & 4u) continue;  // not active, or joined meanwhile
            atomicXor(&S32[jn[d] >> 2], 2u << sh);
            append((int)(((uint32_t)cof(d) << 29) | ((uint32_t)zof(d) << 20) |
                         ((uint32_t)yof(d) << 11) | ((uint32_t)xof(d) << 2) |
                         ((old[d] >> sh) & 3u)));
        }
}

// Grid: the lattices at temperature slots [slot0, slot0 + gridDim.x / (CS nconf)) of the group's
// nconf configurations, slot-major (coldest slots first: their clusters are the largest, so they
// start in the first wave), CS CTAs each.  BITS: every bond's activation was decided beforehand
// by wolff_bits_kernel (act, one byte per site: bit b for the site's owned bond b), so a
// frontier site reads bits instead of drawing Philox words and evaluating weights.
template <class Real, bool MASKS, int CS, bool BITS>
__global__ void __launch_bounds__(kGrowThreads, 1)
    wolff_grow_kernel(SweepArgs a, int* list, long long list_stride, long long* csize, int slot0,
                      int nconf, const uint8_t* act, long long act_stride)
{
    const Geo g = a.g;
    int rank = 0;
    if constexpr (CS > 1) rank = (int)cg::this_cluster().block_rank();
    const int lb = (int)blockIdx.x / CS;
    const int slot = slot0 + lb / nconf, conf = lb % nconf;
    const int rep = a.rep_at_temp[conf * a.nrep + slot];
    const int lat = conf * a.nrep + rep;
    const int tid = (int)threadIdx.x, NT = (int)blockDim.x;
    const int gt = rank * NT + tid, GT = CS * NT;  // this thread among the lattice's threads
    uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    uint32_t* S32 = reinterpret_cast<uint32_t*>(S);
    const Real* P = wfield<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    int* Q = list + (long long)lat * list_stride;
    __shared__ int ring_own[kGrowRing];
    __shared__ int ctl_own[5];
    int* ring = ring_own;  // the first CTA's ring and counters
    int* ctl = ctl_own;
    if constexpr (CS > 1) {
        cg::cluster_group cl = cg::this_cluster();
        ring = cl.map_shared_rank(ring_own, 0);
        ctl = cl.map_shared_rank(ctl_own, 0);
    }
    auto sync_all = []() {
        if constexpr (CS > 1)
            cg::this_cluster().sync();
        else
            __syncthreads();
    };

    const uint32_t cycle = a.ctl[0];
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    if (rank == 0 && tid == 0) {
        const uint32_t w =
            philox4x32_10((uint32_t)rep, cycle, 0xFFFFFFFFu, kTagWolffSeed, k0, k1).x;
        const int seed_site = (int)(((unsigned long long)w * (unsigned long long)g.N) >> 32);
        const int cs = compact_of_site(g, seed_site);
        ctl_own[kCtlHead] = ctl_own[kCtlEnd] = ctl_own[kCtlTail] = 0;
        ctl_own[kCtlRlim] = ctl_own[kCtlWlim] = kGrowRing;
        const int b = S[cs];
        if (b != 1) {  // a vacant seed flips nothing
            S[cs] = (uint8_t)((2 - b) | 4);
            const int x = seed_site % g.L, y = (seed_site / g.L) % g.L, z = seed_site / (g.L * g.L);
            const int cc = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
            Q[0] = ring_own[0] = (int)(((uint32_t)cc << 29) | ((uint32_t)(z >> 1) << 20) |
                                       ((uint32_t)(y >> 1) << 11) | ((uint32_t)(x >> 1) << 2) |
                                       (uint32_t)b);
            ctl_own[kCtlEnd] = ctl_own[kCtlTail] = 1;
        }
    }
    sync_all();

    const double beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
    const float kbw = trial_scale(beta);
    Real J2, J3;
    if constexpr (sizeof(Real) == 8) {
        J2 = a.J2;
        J3 = a.J3;
    } else {
        J2 = a.J2f;
        J3 = a.J3f;
    }
    const unsigned long long thr2 = uniform_threshold<Real>(J2 < Real(0) ? -J2 : J2, beta);
    const unsigned long long thr3 = uniform_threshold<Real>(J3 < Real(0) ? -J3 : J3, beta);
    const int s2 = J2 > Real(0) ? 1 : J2 < Real(0) ? -1 : 0;  // s_i s_j of a satisfied bond
    const int s3 = J3 > Real(0) ? 1 : J3 < Real(0) ? -1 : 0;
    GrowLattice gl;
    gl.S = S;
    gl.S32 = S32;
    gl.A = BITS ? act + (long long)lat * act_stride : nullptr;
    gl.rep = rep;
    gl.cycle = cycle;
    gl.k0 = k0;
    gl.k1 = k1;
    gl.beta = beta;
    gl.kb = kbw;
    gl.thr2 = thr2;
    gl.thr3 = thr3;
    gl.s2 = s2;
    gl.s3 = s3;

    for (int level = 0; level < g.N; ++level) {  // at most N levels: every site joins once
        const int head = ctl[kCtlHead], end = ctl[kCtlEnd], rlim = ctl[kCtlRlim],
                  wlim = ctl[kCtlWlim];
        if (head == end) break;
        auto append = [&](int entry) {
            const int pos = atomicAdd(&ctl[kCtlTail], 1);
            Q[pos] = entry;
            if (pos < wlim) ring[pos & (kGrowRing - 1)] = entry;
        };
        for (int idx = head + gt; idx < end; idx += GT) {
            // entry: compact coordinates and original spin byte of a cluster site
            const uint32_t e = (uint32_t)(idx < rlim ? ring[idx & (kGrowRing - 1)] : Q[idx]);
            grow_entry<Real, MASKS, BITS>(a, g, P, BM, gl, e, append);
        }
        sync_all();
        if (rank == 0 && tid == 0) {
            ctl_own[kCtlRlim] = wlim;
            ctl_own[kCtlHead] = end;
            ctl_own[kCtlEnd] = ctl_own[kCtlTail];
            ctl_own[kCtlWlim] = end + kGrowRing;
        }
        sync_all();
    }
    // clear the join bits of the cluster; atomically, at L2, where the flips were made (a plain
    // read-modify-write could see a line cached before the flip); the list goes back to empty
    // entries for the next update
    const int n = ctl[kCtlTail];
    for (int k = gt; k < n; k += GT) {
        const uint32_t e = (uint32_t)Q[k];
        const int i = cidx(g, (int)(e >> 29), (int)((e >> 20) & 511), (int)((e >> 11) & 511),
                           (int)((e >> 2) & 511));
        atomicAnd(&S32[i >> 2], ~(4u << (8 * (i & 3))));
        Q[k] = kGrowEmpty;
    }
    if (rank == 0 && tid == 0) csize[lat] += n;
    if constexpr (CS > 1) cg::this_cluster().sync();  // the first CTA's counters were read above
}

template <class Real, bool MASKS, int CS, bool BITS>
cudaError_t grow_launch(const SweepArgs& a, int nconf, int slot0, int nslots, int* list,
                        long long list_stride, long long* csize, const uint8_t* act,
                        long long act_stride, cudaStream_t st)
{
    auto kern = wolff_grow_kernel<Real, MASKS, CS, BITS>;
    const int nlat = nconf * nslots;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nlat * CS));
    cfg.blockDim = dim3(kGrowThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)CS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = CS > 1 ? 1u : 0u;
    return cudaLaunchKernelEx(&cfg, kern, a, list, list_stride, csize, slot0, nconf, act,
                              act_stride);
}

template <class Real, bool MASKS, int CS>
int grow_fits()
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)CS);
    cfg.blockDim = dim3(kGrowThreads);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)CS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, wolff_grow_kernel<Real, MASKS, CS, false>, &cfg) !=
        cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return n;
}

// ---- level-free seed-cluster growth ------------------------------------------------------------
// The flipped cluster is the seed's component of the activated-bond graph whatever the order in
// which its sites are processed: a bond's activation depends only on its owner's Philox word and
// on the configuration before the update (a site's byte keeps its original spin until the site
// is claimed, and the claim, an atomic OR, precedes the flip), and every activated bond from a
// claimed site to an unclaimed one claims the latter.  So this form has no levels: each thread
// takes the next queued site as soon as one is queued, and no thread waits for a level's slowest
// site at a barrier (the level-synchronous form's top stall on the coldest lattices).
//   Queue: a new site's entry goes to the global list at a position from a shared counter and to
// a shared-memory ring as a (position, entry) pair; the taker of position p reads the ring slot,
// or the list if a later position has overwritten the slot (the list holds empty entries before
// the update, and position p is written once, right after it is reserved).
//   Termination: a thread whose position is beyond every reserved one stops once every reserved
// site has been processed; a site's reservations precede its completion count (a fence orders
// them), so no site can still be queued then.
//   Every wait is bounded: a wait that gives up sets the context's error word and stops the
// growth (the host reports J1J2C_ETIMEOUT and refills the list with empty entries).
constexpr int kAsyncRing = 8192;    // ring slots: 64 KiB of dynamic shared memory
constexpr int kAsyncWait = 1 << 22; // polls of one wait before it gives up

enum : int { kAsyncTail = 0, kAsyncTaken = 1, kAsyncDone = 2, kAsyncFail = 3 };

__device__ __forceinline__ int vload(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

__device__ __forceinline__ unsigned long long vload64(const unsigned long long* p)
{
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

// Grid: the lattices at temperature slots [slot0, slot0 + gridDim.x / nconf) of the group's nconf
// configurations, slot-major (coldest first), one CTA each
template <class Real, bool MASKS>
__global__ void __launch_bounds__(kGrowThreads, 1)
    wolff_grow_async_kernel(SweepArgs a, int* list, long long list_stride, long long* csize,
                            int slot0, int nconf)
{
    extern __shared__ __align__(16) unsigned long long aring[];
    __shared__ int ctl[4];
    const Geo g = a.g;
    const int lb = (int)blockIdx.x;
    const int slot = slot0 + lb / nconf, conf = lb % nconf;
    const int rep = a.rep_at_temp[conf * a.nrep + slot];
    const int lat = conf * a.nrep + rep;
    const int tid = (int)threadIdx.x, NT = (int)blockDim.x;
    uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    uint32_t* S32 = reinterpret_cast<uint32_t*>(S);
    const Real* P = wfield<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    int* Q = list + (long long)lat * list_stride;
    for (int k = tid; k < kAsyncRing; k += NT) aring[k] = ~0ull;  // no position
    const uint32_t cycle = a.ctl[0];
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    __syncthreads();
    if (tid == 0) {
        const uint32_t w =
            philox4x32_10((uint32_t)rep, cycle, 0xFFFFFFFFu, kTagWolffSeed, k0, k1).x;
        const int seed_site = (int)(((unsigned long long)w * (unsigned long long)g.N) >> 32);
        const int cs = compact_of_site(g, seed_site);
        ctl[kAsyncTail] = ctl[kAsyncTaken] = ctl[kAsyncDone] = ctl[kAsyncFail] = 0;
        const int b = S[cs];
        if (b != 1) {  // a vacant seed flips nothing
            S[cs] = (uint8_t)((2 - b) | 4);
            const int x = seed_site % g.L, y = (seed_site / g.L) % g.L, z = seed_site / (g.L * g.L);
            const int cc = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
            const int entry = (int)(((uint32_t)cc << 29) | ((uint32_t)(z >> 1) << 20) |
                                    ((uint32_t)(y >> 1) << 11) | ((uint32_t)(x >> 1) << 2) |
                                    (uint32_t)b);
            Q[0] = entry;
            aring[0] = (unsigned long long)(uint32_t)entry;  // position 0
            ctl[kAsyncTail] = 1;
        }
    }
    __syncthreads();

    const double beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
    const float kbw = trial_scale(beta);
    Real J2, J3;
    if constexpr (sizeof(Real) == 8) {
        J2 = a.J2;
        J3 = a.J3;
    } else {
        J2 = a.J2f;
        J3 = a.J3f;
    }
    GrowLattice gl;
    gl.S = S;
    gl.S32 = S32;
    gl.A = nullptr;
    gl.rep = rep;
    gl.cycle = cycle;
    gl.k0 = k0;
    gl.k1 = k1;
    gl.beta = beta;
    gl.kb = kbw;
    gl.thr2 = uniform_threshold<Real>(J2 < Real(0) ? -J2 : J2, beta);
    gl.thr3 = uniform_threshold<Real>(J3 < Real(0) ? -J3 : J3, beta);
    gl.s2 = J2 > Real(0) ? 1 : J2 < Real(0) ? -1 : 0;
    gl.s3 = J3 > Real(0) ? 1 : J3 < Real(0) ? -1 : 0;
    auto append = [&](int entry) {
        const int pos = atomicAdd(&ctl[kAsyncTail], 1);
        Q[pos] = entry;
        *reinterpret_cast<volatile unsigned long long*>(&aring[pos & (kAsyncRing - 1)]) =
            ((unsigned long long)(uint32_t)pos << 32) | (uint32_t)entry;
    };
    for (;;) {
        const int idx = atomicAdd(&ctl[kAsyncTaken], 1);
        // wait until position idx is reserved, or until nothing can be queued any more
        bool have = false;
        for (int it = 0;; ++it) {
            if (idx < vload(&ctl[kAsyncTail])) {
                have = true;
                break;
            }
            const int done = vload(&ctl[kAsyncDone]);
            __threadfence_block();
            if (done == vload(&ctl[kAsyncTail]) || vload(&ctl[kAsyncFail])) break;
            if (it >= kAsyncWait) {
                atomicExch(&ctl[kAsyncFail], 1);
                break;
            }
            __nanosleep(64);
        }
        if (!have) break;
        // the entry at position idx: the ring slot, else the list once it is written
        uint32_t e = 0;
        bool got = false;
        for (int it = 0; it < kAsyncWait; ++it) {
            const unsigned long long v = vload64(&aring[idx & (kAsyncRing - 1)]);
            if ((uint32_t)(v >> 32) == (uint32_t)idx) {
                e = (uint32_t)v;
                got = true;
                break;
            }
            const int q = vload(&Q[idx]);
            if (q != kGrowEmpty) {
                e = (uint32_t)q;
                got = true;
                break;
            }
            __nanosleep(32);
        }
        if (got) grow_entry<Real, MASKS, false>(a, g, P, BM, gl, e, append);
        else atomicExch(&ctl[kAsyncFail], 1);
        __threadfence_block();  // this site's reservations before its completion
        atomicAdd(&ctl[kAsyncDone], 1);
    }
    __syncthreads();
    // clear the join bits of the cluster (atomically, at L2, where the flips were made) and
    // empty the list for the next update; every reserved position was written before its
    // reserving thread counted its site done
    const int n = ctl[kAsyncTail];
    for (int k = tid; k < n; k += NT) {
        const uint32_t e = (uint32_t)vload(&Q[k]);
        if (e == (uint32_t)kGrowEmpty) continue;
        const int i = cidx(g, (int)(e >> 29), (int)((e >> 20) & 511), (int)((e >> 11) & 511),
                           (int)((e >> 2) & 511));
        atomicAnd(&S32[i >> 2], ~(4u << (8 * (i & 3))));
        Q[k] = kGrowEmpty;
    }
    if (tid == 0) {
        csize[lat] += n;
        if (ctl[kAsyncFail] && a.err) atomicExch(a.err, 1);
    }
}

template <class Real, bool MASKS>
cudaError_t grow_async_launch(const SweepArgs& a, int nconf, int slot0, int nslots, int* list,
                              long long list_stride, long long* csize, cudaStream_t st)
{
    auto kern = wolff_grow_async_kernel<Real, MASKS>;
    const size_t smem = sizeof(unsigned long long) * kAsyncRing;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<nconf * nslots, kGrowThreads, smem, st>>>(a, list, list_stride, csize, slot0, nconf);
    return cudaGetLastError();
}

// act: the activation bits of wolff_bits_kernel (one CTA per lattice), or nullptr
template <class Real, bool MASKS>
cudaError_t grow_dispatch(const SweepArgs& a, int nconf, int slot0, int nslots, int cs, int* list,
                          long long list_stride, long long* csize, const uint8_t* act,
                          long long act_stride, cudaStream_t st)
{
    if (act)
        return grow_launch<Real, MASKS, 1, true>(a, nconf, slot0, nslots, list, list_stride,
                                                 csize, act, act_stride, st);
    if (cs < 0)
        return grow_async_launch<Real, MASKS>(a, nconf, slot0, nslots, list, list_stride, csize,
                                              st);
    if (cs == 2)
        return grow_launch<Real, MASKS, 2, false>(a, nconf, slot0, nslots, list, list_stride,
                                                  csize, nullptr, 0, st);
    if (cs == 4)
        return grow_launch<Real, MASKS, 4, false>(a, nconf, slot0, nslots, list, list_stride,
                                                  csize, nullptr, 0, st);
    return grow_launch<Real, MASKS, 1, false>(a, nconf, slot0, nslots, list, list_stride, csize,
                                              nullptr, 0, st);
}

// Activation of every site's five owned bonds (+x, +y, (+x,+y), (-x,+y), +z) for the next Wolff
// update, decided exactly as the growth kernel decides them when it reaches the bond (the
// owner's Philox word, K s_i s_j > 0 from the configuration before the flip, the same
// arithmetic): bit b of act[i].  One thread per Philox quad group of four sites; grid (quad
// groups / 256, lattices at temperature slots [slot0, ...) of the nconf configurations,
// slot-major like the growth grid).  Every site is evaluated whether or not the cluster reaches
// it, so this pays where the cluster spans most of the lattice (the cold slots), and it runs on
// every SM instead of the one that grows the cluster.
template <class Real, bool MASKS>
__global__ void __launch_bounds__(256) wolff_bits_kernel(SweepArgs a, uint8_t* act,
                                                         long long act_stride, int slot0, int nconf)
{
    const Geo g = a.g;
    const int lb = (int)blockIdx.y;
    const int slot = slot0 + lb / nconf, conf = lb % nconf;
    const int rep = a.rep_at_temp[conf * a.nrep + slot];
    const int lat = conf * a.nrep + rep;
    const int q = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (q >= 8 * g.Hh * g.Lh * g.Qr) return;
    int r = q;
    const int Xq = r % g.Qr;
    r /= g.Qr;
    const int Y = r % g.Lh;
    r /= g.Lh;
    const int Z = r % g.Hh, c = r / g.Hh;
    const int X0 = 4 * Xq, nw = g.Lh - X0 < 4 ? g.Lh - X0 : 4;
    const int px = c & 1, py = (c >> 1) & 1, pz = c >> 2;
    const uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    const Real* P = wfield<Real>(a, conf);
    const uint8_t* BM = MASKS ? a.bm + (long long)conf * a.lat_stride : nullptr;
    uint8_t* A = act + (long long)lat * act_stride;
    const uint32_t cycle = a.ctl[0];
    const uint32_t k0 = a.seed, k1 = a.conf_base + (uint32_t)conf;
    const double beta = a.beta[conf * a.nrep + a.temp_of_rep[conf * a.nrep + rep]];
    const float kbw = trial_scale(beta);
    Real J2, J3;
    if constexpr (sizeof(Real) == 8) {
        J2 = a.J2;
        J3 = a.J3;
    } else {
        J2 = a.J2f;
        J3 = a.J3f;
    }
    const unsigned long long thr2 = uniform_threshold<Real>(J2 < Real(0) ? -J2 : J2, beta);
    const unsigned long long thr3 = uniform_threshold<Real>(J3 < Real(0) ? -J3 : J3, beta);
    const int s2 = J2 > Real(0) ? 1 : J2 < Real(0) ? -1 : 0;  // s_i s_j of a satisfied bond
    const int s3 = J3 > Real(0) ? 1 : J3 < Real(0) ? -1 : 0;
    const int Yp = py ? (Y + 1 == g.Lh ? 0 : Y + 1) : Y;
    const int Zp = pz ? (Z + 1 == g.Hh ? 0 : Z + 1) : Z;
    // the +z bonds' words: one call for the quad group (word X & 3)
    const U4 zw = philox4x32_10((uint32_t)rep, cycle, (uint32_t)q, kTagWolffZ, k0, k1);
    uint32_t out = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        if (w >= nw) break;
        const int X = X0 + w;
        const int i = cidx(g, c, Z, Y, X);
        const int si = (S[i] & 3) - 1;
        if (si == 0) continue;  // a vacancy owns no bond
        const int Xp = px ? (X + 1 == g.Lh ? 0 : X + 1) : X;
        const int Xm = px ? X : (X == 0 ? g.Lh - 1 : X - 1);
        int jn[5];
        jn[0] = cidx(g, c ^ 1, Z, Y, Xp);
        jn[1] = cidx(g, c ^ 2, Z, Yp, X);
        jn[2] = cidx(g, c ^ 3, Z, Yp, Xp);
        jn[3] = cidx(g, c ^ 3, Z, Yp, Xm);
        jn[4] = cidx(g, c ^ 4, Zp, Y, X);
        int sj[5];
#pragma unroll
        for (int b = 0; b < 5; ++b) sj[b] = (S[jn[b]] & 3) - 1;
        const U4 own = philox4x32_10((uint32_t)rep, cycle, (uint32_t)i, kTagWolffSite, k0, k1);
        int m = 3;
        if (MASKS) m = BM[i];
        unsigned bits = 0;
#pragma unroll
        for (int b = 0; b < 5; ++b) {
            if (sj[b] == 0) continue;
            bool on;
            if (b < 2) {
                Real wv;
                on = bond_weight<Real>(a, b, si, sj[b], m & 1, (m >> 1) & 1, P[i], P[jn[b]],
                                       wv) &&
                     bond_trial<Real>(wv, beta, kbw, u4_word(own, b));
            } else {
                on = si * sj[b] == (b < 4 ? s2 : s3) &&
                     uniform_trial<Real>(b < 4 ? thr2 : thr3, b < 4 ? u4_word(own, b)
                                                                    : u4_word(zw, X & 3));
            }
            if (on) bits |= 1u << b;
        }
        out |= bits << (8 * w);
    }
    const int i0 = cidx(g, c, Z, Y, X0);
    if (nw == 4 && (i0 & 3) == 0) {
        *reinterpret_cast<uint32_t*>(A + i0) = out;
    } else {
        for (int w = 0; w < nw; ++w) A[i0 + w] = (uint8_t)(out >> (8 * w));
    }
}

template <class Real>
cudaError_t bonds(const SweepArgs& a, int* labels, long long ls, int* err, int nlat, bool masks,
                  cudaStream_t st)
{
    dim3 grid((unsigned)((a.g.N + 255) / 256), (unsigned)nlat);
    if (masks)
        wolff_bond_kernel<Real, true><<<grid, 256, 0, st>>>(a, labels, ls, err);
    else
        wolff_bond_kernel<Real, false><<<grid, 256, 0, st>>>(a, labels, ls, err);
    return cudaGetLastError();
}

}  // namespace

// The growth form for the lattices at temperature slots [slot0, slot0 + nslots) of the group's
// nconf configurations, cs CTAs per lattice
cudaError_t launch_wolff_grow(const SweepArgs& a, bool fp64, bool masks, int nconf, int slot0,
                              int nslots, int cs, int* labels, long long lab_stride,
                              long long* csize, cudaStream_t st, const uint8_t* act,
                              long long act_stride)
{
    if (nslots <= 0) return cudaSuccess;
    if (fp64)
        return masks ? grow_dispatch<double, true>(a, nconf, slot0, nslots, cs, labels,
                                                   lab_stride, csize, act, act_stride, st)
                     : grow_dispatch<double, false>(a, nconf, slot0, nslots, cs, labels,
                                                    lab_stride, csize, act, act_stride, st);
    return masks ? grow_dispatch<float, true>(a, nconf, slot0, nslots, cs, labels, lab_stride,
                                              csize, act, act_stride, st)
                 : grow_dispatch<float, false>(a, nconf, slot0, nslots, cs, labels, lab_stride,
                                               csize, act, act_stride, st);
}

cudaError_t launch_wolff_bits(const SweepArgs& a, bool fp64, bool masks, int nconf, int slot0,
                              int nslots, uint8_t* act, long long act_stride, cudaStream_t st)
{
    if (nslots <= 0) return cudaSuccess;
    const int nq = 8 * a.g.Hh * a.g.Lh * a.g.Qr;
    const dim3 grid((unsigned)((nq + 255) / 256), (unsigned)(nconf * nslots));
    if (fp64) {
        if (masks)
            wolff_bits_kernel<double, true><<<grid, 256, 0, st>>>(a, act, act_stride, slot0, nconf);
        else
            wolff_bits_kernel<double, false><<<grid, 256, 0, st>>>(a, act, act_stride, slot0,
                                                                   nconf);
    } else {
        if (masks)
            wolff_bits_kernel<float, true><<<grid, 256, 0, st>>>(a, act, act_stride, slot0, nconf);
        else
            wolff_bits_kernel<float, false><<<grid, 256, 0, st>>>(a, act, act_stride, slot0,
                                                                  nconf);
    }
    return cudaGetLastError();
}

// Clusters of cs CTAs (2 or 4) of the growth kernel that can be resident at once (0: none)
int wolff_grow_clusters(bool fp64, bool masks, int cs)
{
    if (cs == 2)
        return fp64 ? (masks ? grow_fits<double, true, 2>() : grow_fits<double, false, 2>())
                    : (masks ? grow_fits<float, true, 2>() : grow_fits<float, false, 2>());
    if (cs == 4)
        return fp64 ? (masks ? grow_fits<double, true, 4>() : grow_fits<double, false, 4>())
                    : (masks ? grow_fits<float, true, 4>() : grow_fits<float, false, 4>());
    return 0;
}

// Planes per slab of the shared-memory form: the largest even divisor pz of H whose slab fits
// kSlabSites2 sites (two CTAs per SM), else kSlabSites1 (one CTA per SM); 0 if none does.
constexpr int kSlabSites2 = 38912, kSlabSites1 = 65536, kSlabThreads = 512;

int wolff_slab_planes(const Geo& g)
{
    for (const int cap : {kSlabSites2, kSlabSites1})
        for (int pz = g.H; pz >= 2; pz -= 2)
            if (g.H % pz == 0 && (long long)pz * g.L * g.L <= cap) return pz;
    return 0;
}

namespace {
template <class Real, bool MASKS>
cudaError_t slab_launch(const SweepArgs& a, int pz, int nlat, int* labels, long long ls, int* err,
                        cudaStream_t st)
{
    const size_t smem = 3 * (size_t)pz * a.g.L * a.g.L;
    // the limit is the most the device allows, valid for every slab size in one context
    cudaError_t e = raise_smem_limit(wolff_slab_kernel<Real, MASKS>);
    if (e != cudaSuccess) return e;
    wolff_slab_kernel<Real, MASKS>
        <<<dim3((unsigned)(a.g.H / pz), (unsigned)nlat), kSlabThreads, smem, st>>>(a, pz, labels,
                                                                                 ls, err);
    if ((e = cudaGetLastError()) != cudaSuccess || pz == a.g.H) return e;
    const int items = (a.g.H / pz) * 4 * a.g.Lh * a.g.Qr;
    wolff_boundary_kernel<Real><<<dim3((unsigned)((items + 255) / 256), (unsigned)nlat), 256, 0,
                                  st>>>(a, pz, labels, ls, err);
    return cudaGetLastError();
}
}  // namespace

// One Wolff update of every lattice of a group (the SweepArgs of the group, lat0 = 0): labels is
// scratch of nlat x lab_stride ints (labels, or the cluster list of the growth form), csize
// receives the flipped-cluster size per lattice (added; the caller zeroes it), err is set on a
// union-find retry overflow.
cudaError_t launch_wolff(const SweepArgs& a, bool fp64, bool masks, int nlat, int* labels,
                         long long lab_stride, long long* csize, int* err, cudaStream_t st,
                         WolffForm form, int grow_cs)
{
    const unsigned bx = (unsigned)((a.g.N + 255) / 256);
    const unsigned bxs = bx > 64 ? 64u : bx;
    cudaError_t e;
    if (form == kWolffGrow) {
        return launch_wolff_grow(a, fp64, masks, nlat / a.nrep, 0, a.nrep, grow_cs, labels,
                                 lab_stride, csize, st);
    }
    const int pz = form == kWolffSlab ? wolff_slab_planes(a.g) : 0;
    if (pz > 0) {
        e = fp64 ? (masks ? slab_launch<double, true>(a, pz, nlat, labels, lab_stride, err, st)
                          : slab_launch<double, false>(a, pz, nlat, labels, lab_stride, err, st))
                 : (masks ? slab_launch<float, true>(a, pz, nlat, labels, lab_stride, err, st)
                          : slab_launch<float, false>(a, pz, nlat, labels, lab_stride, err, st));
    } else {
        wolff_init_kernel<<<dim3(bxs, (unsigned)nlat), 256, 0, st>>>(labels, lab_stride, a.g.N);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        e = fp64 ? bonds<double>(a, labels, lab_stride, err, nlat, masks, st)
                 : bonds<float>(a, labels, lab_stride, err, nlat, masks, st);
    }
    if (e != cudaSuccess) return e;
    wolff_flip_kernel<<<dim3(bxs, (unsigned)nlat), 256, 0, st>>>(a, labels, lab_stride, csize);
    return cudaGetLastError();
}

}  // namespace j1j2
