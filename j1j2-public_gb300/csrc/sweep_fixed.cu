// Shape-specialised sweep kernel: the lattice extents (L/2, H/2) and the CTA size are template
// constants and the eight colour phases of a sweep are unrolled, so colour parities are
// compile-time.  Each thread owns the same quad(s) in every colour class; the word offsets of the
// quad's neighbours inside a colour block are computed once, and a colour phase addresses shared
// memory as [offset + colour base], the base being an immediate.  With two quads per thread both
// quads' operands are loaded before either is updated (quads of one colour never neighbour each
// other), which doubles the instruction-level parallelism of a thread.  Same arithmetic, Philox
// stream and outputs as the generic quad kernel (kernels.cu), bit for bit.  One CTA owns one
// lattice, staged in shared memory for the PTSWAPEVER fused sweeps of a PT cycle.
#include "quad_sweep.cuh"

namespace j1j2 {
namespace {

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

// The same kernel over R replicas of one configuration per CTA (colour_phase_r / all_colours_r
// of quad_sweep.cuh): results are those of sweep_fixed_kernel bit for bit.
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
    extern __shared__ __align__(128) unsigned char ssmem[];  // 128-aligned bulk-copy buffers
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
        stream_copy_in<Real, LH, HH>(ssmem + Lay::PB, a.spins + (long long)lat * a.lat_stride,
                                     Lay::SB, &bar[0]);
        stream_copy_in<Real, LH, HH>(ssmem, field_base<Real>(a, lat / a.nrep), Lay::PB, &bar[2]);
        st = StreamState{0u, 1u | 4u, 1, 0};
    }
    OffsetCache<QPT> off;
    fill_offsets<LH, HH, NT, QPT>(off, tid);
    // (the first step's barrier publishes thread 0's initialisation)
#pragma unroll 1
    for (int l = first; l < last; l += 2) {
        if (!stream_step<Real, LH, HH, NT, QPT, VAC, 0>(a, ssmem, bar, &st, off, l, last)) break;
        if (l + 1 < last &&
            !stream_step<Real, LH, HH, NT, QPT, VAC, 1>(a, ssmem, bar, &st, off, l + 1, last))
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

}  // namespace j1j2
