// One persistent launch over every lattice-shape group of a context (the mixed-L batch): a CTA
// per SM takes tiles from one queue until it is empty, so the shapes share the SMs without a
// kernel boundary between them, and the largest tiles go first.  A tile is R replicas of one
// configuration side by side in shared memory behind one staged copy of their field (the L = 48
// field stays in L2): two lattices of 32^3, three of 24^3, eight of 16^3 (four thread groups of
// two, each group a whole colour class per phase), or one of 48^3.  Every tile runs the same
// quad arithmetic, Philox words and colour order as the one-lattice kernels (quad_sweep.cuh), so
// the results are theirs bit for bit.
#include "quad_sweep.cuh"

namespace j1j2 {
namespace {

constexpr int kMultiThreads = 512;

// Tile shapes: LH, HH, thread groups G of NTG threads each (the CTA's other threads only meet
// the barriers), replicas per thread group, field staged.  The L = 48 tile runs 432 threads, three
// z-planes of quads: each takes eight quads one plane-stride apart, whose offsets are the
// first one's shifted (no recomputation per colour phase).
template <int K>
struct Tile;
template <>
struct Tile<0> {  // L = 16
    static constexpr int LH = 8, HH = 8, G = 4, NTG = kMultiThreads / 4, RG = 2;
    static constexpr bool STAGE = true;
};
template <>
struct Tile<1> {  // L = 24
    static constexpr int LH = 12, HH = 12, G = 1, NTG = kMultiThreads, RG = 3;
    static constexpr bool STAGE = true;
};
template <>
struct Tile<2> {  // L = 32
    static constexpr int LH = 16, HH = 16, G = 1, NTG = kMultiThreads, RG = 2;
    static constexpr bool STAGE = true;
};
template <>
struct Tile<3> {  // L = 48
    static constexpr int LH = 24, HH = 24, G = 1, NTG = 432, RG = 1;
    static constexpr bool STAGE = false;
};
template <int K>
constexpr size_t tile_smem()
{
    using T = Tile<K>;
    using Sh = Shape<T::LH, T::HH>;
    return (size_t)(T::G * T::RG) * Sh::NB + (T::STAGE ? (size_t)Sh::N * sizeof(float) : 0);
}

// One tile: the lattices lat0 .. lat0 + R - 1 of group gd (replicas of one configuration)
template <int K, bool VAC>
__device__ __forceinline__ void multi_tile(const SweepArgs& a, const GroupDesc& gd, int lat0,
                                           unsigned char* smem)
{
    using T = Tile<K>;
    constexpr int LH = T::LH, HH = T::HH, G = T::G, RG = T::RG, R = G * RG;
    using Sh = Shape<LH, HH>;
    constexpr int NTG = T::NTG;  // threads per thread group
    constexpr int QPT = (Sh::CS + NTG - 1) / NTG;
    static_assert(G * NTG <= kMultiThreads, "thread groups exceed the CTA");
    // several thread groups only where each takes a whole colour class per phase (the colour
    // phases then never test threadIdx.x against the quad count)
    static_assert(G == 1 || QPT * NTG == Sh::CS, "thread groups must cover a colour exactly");
    const int grp = (int)threadIdx.x / NTG, tl = (int)threadIdx.x - grp * NTG;
    const bool active = grp < G;
    const int cl = lat0 / gd.nrep;    // configuration within the group
    const int conf = gd.conf0 + cl;   // within the context: Philox key word 1 = conf_base + conf
    const float* Pg = gd.pf + (long long)cl * gd.p_stride;
    float* Ps = reinterpret_cast<float*>(smem + R * Sh::NB);
#pragma unroll
    for (int r = 0; r < R; ++r)
        block_copy16(smem + r * Sh::NB, gd.spins + (long long)(lat0 + r) * gd.lat_stride, Sh::NB);
    if constexpr (T::STAGE)
        block_copy16_ldg(Ps, Pg, (int)((Sh::N * sizeof(float) + 15) & ~(size_t)15));
    OffsetCache<QPT> off;
    fill_offsets<LH, HH, NTG, QPT>(off, tl);
    __syncthreads();
    const float* P = T::STAGE ? Ps : Pg;
    uint32_t* S32[RG];
    int rep[RG];
    double beta[RG];
    float kb[RG];
    Acc acc[RG];
#pragma unroll
    for (int j = 0; j < RG; ++j) {
        const int r = (active ? grp : 0) * RG + j;
        S32[j] = reinterpret_cast<uint32_t*>(smem + r * Sh::NB);
        rep[j] = lat0 + r - cl * gd.nrep;
        beta[j] = a.use_override ? a.beta_override
                                 : gd.beta[cl * gd.nrep + gd.tor[cl * gd.nrep + rep[j]]];
        kb[j] = (float)(-2.0 * beta[j] * 1.4426950408889634);
        acc[j] = Acc{0, 0, 0, 0, 0};
    }
    const uint32_t sweep0 =
        a.use_override ? a.sweep_override : a.ctl[0] * (uint32_t)a.ptswapever;
#pragma unroll 1
    for (int t = 0; t < a.nsweeps; ++t)
        all_colours_r<float, LH, HH, NTG, QPT, RG, false, VAC>(
            a, S32, P, off, sweep0 + (uint32_t)t, rep, (uint32_t)conf, beta, kb, acc, active);
    all_colours_r<float, LH, HH, NTG, QPT, RG, true, VAC>(a, S32, P, off, 0u, rep,
                                                          (uint32_t)conf, beta, kb, acc, active);
    // replica r's sums are held by thread group r / RG; the others (and inactive threads) add
    // zeros
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const Acc v = r / RG == grp ? acc[r % RG] : Acc{0, 0, 0, 0, 0};
        const Acc tot = block_reduce(v);
        if (threadIdx.x == 0) store_obs(gd.obs + lat0 + r, tot);
        __syncthreads();  // block_reduce's scratch is reused by the next replica
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
        block_copy16(gd.spins + (long long)(lat0 + r) * gd.lat_stride, smem + r * Sh::NB,
                     Sh::NB);
}

// Grid: at most one CTA per SM; each takes the next task of m.tasks until the queue is empty
// (m.queue[0] is zero at the launch)
template <bool VAC>
__global__ void __launch_bounds__(kMultiThreads, 1) sweep_multi_kernel(MultiArgs m)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int task;
    for (;;) {
        if (threadIdx.x == 0) task = (int)atomicAdd(m.queue, 1u);
        __syncthreads();
        const int t = task;  // the same in every thread: thread 0 writes it again only after the
                             // barrier that ends this tile
        if (t >= m.ntasks) break;
        const int2 tk = m.tasks[t];
        const GroupDesc gd = m.groups[tk.x];
        switch (gd.kind) {
            case 0:
                multi_tile<0, VAC>(m.a, gd, tk.y, smem);
                break;
            case 1:
                multi_tile<1, VAC>(m.a, gd, tk.y, smem);
                break;
            case 2:
                multi_tile<2, VAC>(m.a, gd, tk.y, smem);
                break;
            default:
                multi_tile<3, VAC>(m.a, gd, tk.y, smem);
                break;
        }
        __syncthreads();  // the tile's shared memory and `task` are reused
    }
}

size_t largest_tile_smem()
{
    size_t b = tile_smem<0>();
    if (tile_smem<1>() > b) b = tile_smem<1>();
    if (tile_smem<2>() > b) b = tile_smem<2>();
    if (tile_smem<3>() > b) b = tile_smem<3>();
    return (b + 15) & ~(size_t)15;
}

}  // namespace

int multi_tile_kind(int L, int H)
{
    if (L != H) return -1;
    switch (L) {
        case 16:
            return 0;
        case 24:
            return 1;
        case 32:
            return 2;
        case 48:
            return 3;
        default:
            return -1;
    }
}

int multi_tile_lattices(int kind)
{
    switch (kind) {
        case 0:
            return Tile<0>::G * Tile<0>::RG;
        case 1:
            return Tile<1>::G * Tile<1>::RG;
        case 2:
            return Tile<2>::G * Tile<2>::RG;
        case 3:
            return Tile<3>::G * Tile<3>::RG;
        default:
            return 0;
    }
}

size_t multi_smem_bytes() { return largest_tile_smem(); }

int multi_threads() { return kMultiThreads; }

cudaError_t launch_multi(const MultiArgs& m, bool vac, int grid, cudaStream_t st, bool prepare)
{
    const size_t smem = largest_tile_smem();
    auto k = vac ? sweep_multi_kernel<true> : sweep_multi_kernel<false>;
    if (prepare) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (grid <= 0 || m.ntasks <= 0) return cudaSuccess;
    k<<<grid, kMultiThreads, smem, st>>>(m);
    return cudaGetLastError();
}

}  // namespace j1j2
