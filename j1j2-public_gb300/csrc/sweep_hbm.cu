// Shape-specialised sweep kernels for lattices in HBM (L = 96; L = 32 as a cross-check shape):
// one launch per colour phase over every lattice of a group, with the per-quad arithmetic of the
// shared-memory kernels (quad_sweep.cuh), so the results are theirs bit for bit.  Kept apart from
// sweep_fixed.cu so that the two translation units compile in parallel.
#include "quad_sweep.cuh"

namespace j1j2 {
namespace {

// ---- lattices in HBM --------------------------------------------------------------------------
// Lattices too large for one CTA's shared memory (L = 96: 864 KiB of spins) keep spins and field
// in HBM / L2 and run one launch per colour phase; the kernel boundary is the barrier between
// colours.  One thread per quad with the same compile-time offsets, operand loads and arithmetic
// as the shared-memory kernels (sweep_fixed.cu), so the results are those of every other kernel
// bit for bit.
// Grid: (quads of a colour / NT, lattices).
// One colour phase of quad o in RPT replicas of one configuration: the field operands are loaded
// once and shared, the spin operands of every replica are loaded before any is updated.
template <class Real, int LH, int HH, int C, int RPT, bool VAC, bool SLOTS>
__device__ __forceinline__ void hbm_phase(const SweepArgs& a, const Real* P, const QuadOff& o,
                                          int conf, const int* rep, int s0, uint32_t sweep)
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
        // the replica's slot (s0 + r in the slot-range form), then FP64 its beta, FP32 the slot's
        // acceptance scale, rounded once from beta on the host (no FP64 operation here)
        double beta = a.beta_override;
        float kb = (float)(-2.0 * a.beta_override * 1.4426950408889634);
        if (!a.use_override) {
            const int sl = SLOTS ? s0 + r : a.temp_of_rep[conf * a.nrep + rep[r]];
            if constexpr (sizeof(Real) == 8)
                beta = a.beta[conf * a.nrep + sl];
            else
                kb = a.kb[conf * a.nrep + sl];
        }
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
    int conf, rep[RPT], s0 = -1;
    if (SLOTS) {
        const int per = a.nslots / RPT;
        conf = a.lat0 / a.nrep + (int)blockIdx.y / per;
        s0 = a.slot0 + ((int)blockIdx.y % per) * RPT;
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
        hbm_phase<Real, LH, HH, C, RPT, VAC, SLOTS>(a, P, o, conf, rep, s0, sweep);           \
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
// SLOTS: block row y covers the temperature slots of the sweep kernel's slot-range form, so each
// half of the split cycle measures its own lattices.
template <class Real, int LH, int HH, int NT, int RPT, bool VAC, bool SLOTS>
__global__ void __launch_bounds__(NT) measure_fixed_hbm_kernel(SweepArgs a)
{
    pdl_wait();
    pdl_release();
    using Sh = Shape<LH, HH>;
    const int q = (int)(blockIdx.x * NT + threadIdx.x);
    int conf, lats[RPT];
    if (SLOTS) {
        const int per = a.nslots / RPT;
        conf = a.lat0 / a.nrep + (int)blockIdx.y / per;
        const int s0 = a.slot0 + ((int)blockIdx.y % per) * RPT;
#pragma unroll
        for (int r = 0; r < RPT; ++r)
            lats[r] = conf * a.nrep + a.rep_at_temp[conf * a.nrep + s0 + r];
    } else {
        const int lat = a.lat0 + (int)blockIdx.y * RPT;
        conf = lat / a.nrep;
#pragma unroll
        for (int r = 0; r < RPT; ++r) lats[r] = lat + r;
    }
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
                reinterpret_cast<const uint32_t*>(a.spins + (long long)lats[r] * a.lat_stride), \
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
            LatObs* ob = a.obs + lats[r];
            atomicAdd(reinterpret_cast<unsigned long long*>(&ob->eacc), (unsigned long long)tot.e);
            atomicAdd(&ob->M, tot.M);
            atomicAdd(&ob->SX, tot.SX);
            atomicAdd(&ob->SY, tot.SY);
            atomicAdd(&ob->NB, tot.NB);
        }
        __syncthreads();  // block_reduce's scratch is reused by the next replica
    }
}

// One launch with RPT replicas per thread: the observables (colour < 0) or one colour phase, of
// whole lattices or (a.nslots > 0) of a slot range of every configuration
template <class Real, int LH, int HH, int NT, int RPT>
cudaError_t run_hbm_r(const SweepArgs& a, int colour, int t, int nlat, cudaStream_t st)
{
    constexpr int CS = Shape<LH, HH>::CS;
    const unsigned gx = (unsigned)((CS + NT - 1) / NT);
    const bool pdl = a.pdl != 0;
    const dim3 b((unsigned)NT);
    if (a.nslots > 0) {  // nlat: whole configurations
        const unsigned gy = (unsigned)(nlat / a.nrep * (a.nslots / RPT));
        if (colour < 0)
            return launch_k(pdl, dim3(gx, gy, 8u), b, 0, st,
                            measure_fixed_hbm_kernel<Real, LH, HH, NT, RPT, true, true>, a);
        return launch_k(pdl, dim3(gx, gy), b, 0, st,
                        sweep_fixed_hbm_kernel<Real, LH, HH, NT, RPT, true, true>, a, colour, t);
    }
    const unsigned gy = (unsigned)(nlat / RPT);
    if (colour < 0)
        return launch_k(pdl, dim3(gx, gy, 8u), b, 0, st,
                        measure_fixed_hbm_kernel<Real, LH, HH, NT, RPT, true, false>, a);
    return launch_k(pdl, dim3(gx, gy), b, 0, st,
                    sweep_fixed_hbm_kernel<Real, LH, HH, NT, RPT, true, false>, a, colour, t);
}

template <class Real, int LH, int HH, int NT>
cudaError_t run_hbm(const SweepArgs& a, int colour, int t, int nlat, int rpt, cudaStream_t st)
{
    if (rpt == 4) return run_hbm_r<Real, LH, HH, NT, 4>(a, colour, t, nlat, st);
    if (rpt == 2) return run_hbm_r<Real, LH, HH, NT, 2>(a, colour, t, nlat, st);
    return run_hbm_r<Real, LH, HH, NT, 1>(a, colour, t, nlat, st);
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
    {false, 96, 96, 128, run_hbm<float, 48, 48, 128>},
    {false, 96, 96, 512, run_hbm<float, 48, 48, 512>},
    {true, 96, 96, 256, run_hbm<double, 48, 48, 256>},
    {false, 32, 32, 256, run_hbm<float, 16, 16, 256>},
    {true, 32, 32, 256, run_hbm<double, 16, 16, 256>},
};

}  // namespace

int fixed_hbm_threads(bool fp64, int L, int H, bool masks, bool int_cpl)
{
    if (masks || (!fp64 && !int_cpl)) return 0;
    for (const auto& e : kHbm)
        if (e.fp64 == fp64 && e.L == L && e.H == H) return e.nt;
    return 0;
}

int fixed_hbm_sizes(bool fp64, int L, int H, int* out, int cap)
{
    int n = 0;
    for (const auto& e : kHbm)
        if (e.fp64 == fp64 && e.L == L && e.H == H && n < cap) out[n++] = e.nt;
    return n;
}

cudaError_t launch_fixed_hbm(const SweepArgs& a, bool fp64, int nt, int colour, int t, int nlat,
                             int rpt, cudaStream_t st)
{
    // replicas per thread only over whole configurations (RPT lattices of one block row share
    // their configuration's field)
    if (rpt > 1 && (a.nrep % rpt != 0 || a.lat0 % a.nrep != 0 || nlat % a.nrep != 0)) rpt = 1;
    if (rpt != 2 && rpt != 4) rpt = 1;
    if (a.nslots > 0) {  // slot ranges: whole configurations, RPT dividing the range
        if (a.lat0 % a.nrep != 0 || nlat % a.nrep != 0 || a.slot0 < 0 ||
            a.slot0 + a.nslots > a.nrep)
            return cudaErrorInvalidValue;
        while (rpt > 1 && a.nslots % rpt != 0) rpt /= 2;
    }
    for (const auto& e : kHbm)
        if (e.fp64 == fp64 && e.L == a.g.L && e.H == a.g.H && (nt <= 0 || e.nt == nt))
            return e.fn(a, colour, t, nlat, rpt, st);
    return cudaErrorInvalidValue;
}

}  // namespace j1j2
