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
// Components are labelled in a scratch array (one int32 per site) by lock-free union-find:
// hooking the larger root under the smaller with atomicCAS, path halving in find; then every
// label is compressed to its root and the seed's component is flipped.
//
// Streams (Philox4x32-10, key = (seed, conf_base + conf)):
//   bond b of the site in group g: ctr = (replica, cycle, g, 3 + 16*b), word X & 3
//   seed site:                     ctr = (replica, cycle, 0xFFFFFFFF, 4), word 0; the site is
//                                  floor(w * N / 2^32) in reference site order; a vacancy seed
//                                  means no flip this cycle (a configuration-independent choice)
#include "sweep_common.cuh"

namespace j1j2 {
namespace {

enum : uint32_t { kTagWolffBond = 3u, kTagWolffSeed = 4u };

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

// Union of the components of a and b; false if the retry budget ran out (set as an error).
__device__ __forceinline__ bool unite(volatile int* lab, int a, int b)
{
    for (int it = 0; it < (1 << 20); ++it) {
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
#pragma unroll
    for (int b = 0; b < 5; ++b) {
        const int cj = nb[b];
        const int sj = (int)S[cj] - 1;
        if (sj == 0) continue;
        const int ss = si * sj;
        bool active;
        if constexpr (sizeof(Real) == 8) {
            double K;
            if (b == 0)
                K = __dadd_rn(__dadd_rn(jh ? a.J1h : 0.0, P[ci]), P[cj]);
            else if (b == 1)
                K = __dsub_rn(__dsub_rn(jv ? a.J1v : 0.0, P[ci]), P[cj]);
            else if (b < 4)
                K = a.J2;
            else
                K = a.J3;
            const double w = ss > 0 ? K : -K;
            if (!(w > 0.0)) continue;
            const uint32_t r = u4_word(
                philox4x32_10((uint32_t)rep, cycle, grp, kTagWolffBond + 16u * b, k0, k1), X & 3);
            const double pa = __dsub_rn(1.0, own_exp(-__dmul_rn(__dmul_rn(2.0, w), beta)));
            active = u01_f64(r) < pa;
        } else {
            float K;
            if (b == 0)
                K = __fadd_rn(__fadd_rn(jh ? a.J1hf : 0.0f, P[ci]), P[cj]);
            else if (b == 1)
                K = __fsub_rn(__fsub_rn(jv ? a.J1vf : 0.0f, P[ci]), P[cj]);
            else if (b < 4)
                K = a.J2f;
            else
                K = a.J3f;
            const float w = ss > 0 ? K : -K;
            if (!(w > 0.0f)) continue;
            const uint32_t r = u4_word(
                philox4x32_10((uint32_t)rep, cycle, grp, kTagWolffBond + 16u * b, k0, k1), X & 3);
            const float kb2 = (float)(-2.0 * beta * 1.4426950408889634);
            const float pa = __fsub_rn(1.0f, ex2_approx(__fmul_rn(kb2, w)));
            active = u01_f32(r) < pa;
        }
        if (active && !unite(lab, ci, cj)) atomicExch(err, 1);
    }
}

__global__ void wolff_compress_kernel(int* labels, long long lab_stride, int N)
{
    volatile int* lab = labels + (long long)blockIdx.y * lab_stride;
    for (int i = (int)(blockIdx.x * blockDim.x + threadIdx.x); i < N;
         i += (int)(gridDim.x * blockDim.x))
        lab[i] = find_root(lab, i);
}

__global__ void wolff_flip_kernel(SweepArgs a, const int* labels, long long lab_stride,
                                  long long* csize)
{
    const Geo g = a.g;
    const int lat = (int)blockIdx.y;
    const int conf = lat / a.nrep, rep = lat - conf * a.nrep;
    uint8_t* S = a.spins + (long long)lat * a.lat_stride;
    const int* lab = labels + (long long)lat * lab_stride;
    const uint32_t w = philox4x32_10((uint32_t)rep, a.ctl[0], 0xFFFFFFFFu, kTagWolffSeed, a.seed,
                                     a.conf_base + (uint32_t)conf).x;
    const int seed_site = (int)(((unsigned long long)w * (unsigned long long)g.N) >> 32);
    const int cs = compact_of_site(g, seed_site);
    int count = 0;
    if (S[cs] != 1) {
        const int root = lab[cs];
        for (int i = (int)(blockIdx.x * blockDim.x + threadIdx.x); i < g.N;
             i += (int)(gridDim.x * blockDim.x))
            if (lab[i] == root) {
                S[i] = (uint8_t)(2 - S[i]);
                ++count;
            }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) count += __shfl_down_sync(0xFFFFFFFFu, count, o);
    if ((threadIdx.x & 31) == 0 && count) atomicAdd((unsigned long long*)(csize + lat), count);
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

// One Wolff update of every lattice of a group (the SweepArgs of the group, lat0 = 0): labels is
// scratch of nlat x lab_stride ints, csize receives the flipped-cluster size per lattice (added;
// the caller zeroes it), err is set on a union-find retry overflow.
cudaError_t launch_wolff(const SweepArgs& a, bool fp64, bool masks, int nlat, int* labels,
                         long long lab_stride, long long* csize, int* err, cudaStream_t st)
{
    const unsigned bx = (unsigned)((a.g.N + 255) / 256);
    const unsigned bxs = bx > 64 ? 64u : bx;
    wolff_init_kernel<<<dim3(bxs, (unsigned)nlat), 256, 0, st>>>(labels, lab_stride, a.g.N);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = fp64 ? bonds<double>(a, labels, lab_stride, err, nlat, masks, st)
             : bonds<float>(a, labels, lab_stride, err, nlat, masks, st);
    if (e != cudaSuccess) return e;
    wolff_compress_kernel<<<dim3(bxs, (unsigned)nlat), 256, 0, st>>>(labels, lab_stride, a.g.N);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    wolff_flip_kernel<<<dim3(bxs, (unsigned)nlat), 256, 0, st>>>(a, labels, lab_stride, csize);
    return cudaGetLastError();
}

}  // namespace j1j2
