// Kernel argument blocks and launchers shared by the kernels (kernels.cu) and the C-ABI host
// code (api.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "device_common.cuh"

namespace j1j2 {

// Per-lattice reduction written by the sweep kernel after its last sweep: exact integer sums and
// the fixed-point energy (sum over occupied sites of llrint(-s_i*field_i * 2^32)).
struct LatObs {
    long long eacc;
    int M, SX, SY, NB;
    int pad[2];
};

enum : int { kModeSweep = 0, kModeAudit = 1 };

struct SweepArgs {
    Geo g;
    uint8_t* spins;          // lattice l at spins + l*lat_stride (biased bytes, compact layout)
    long long lat_stride;    // bytes, multiple of 16
    const float* pf;         // conf c at pf + c*p_stride (compact), FP32 random field
    const double* pd;        // conf c at pd + c*p_stride (compact), FP64 random field
    const uint8_t* bm;       // conf c at bm + c*lat_stride: bit0 = jh, bit1 = jv (or nullptr)
    long long p_stride;      // elements, multiple of 4
    const double* beta;      // [nconf*nrep], by slot
    const float* kb;         // [nconf*nrep], by slot: (float)(-2 beta log2(e)), the FP32 form's
                             // acceptance scale, rounded once on the host from beta
    const int* temp_of_rep;  // [nconf*nrep]
    const int* rep_at_temp;  // [nconf*nrep]
    const uint32_t* ctl;     // ctl[0] = PT cycle counter
    LatObs* obs;             // [nlat]
    unsigned long long* audit;  // [2]: attempts, mismatches (audit mode)
    double J1h, J1v, J2, J3;
    float J1hf, J1vf, J2f, J3f;
    // integer J2, J3 (|J| <= 8; the FP32 shape-specialised kernels need them): per byte lane,
    // J3*z + J2*d + ij_bias (z, d the biased byte sums of the inter-layer and diagonal spins) is
    // J3*Zs + J2*D + ij_off - 2^23, each lane within 0..255
    int J2i, J3i;
    uint32_t ij_bias;  // 0x01010101 * (4|J3| + 8|J2|)
    float ij_off;      // 2^23 + 4|J3| + 8|J2| + 2 J3 + 4 J2
    int nrep;
    int nsweeps;             // sweeps per launch
    int ptswapever;          // sweep counter = cycle*ptswapever (+ sweep within the cycle)
    uint32_t seed, conf_base;
    // Philox key schedule of the sweep stream: round r of configuration conf uses key words
    // rk0[r] = seed + r * 0x9E3779B9 and rk1[r] + conf = conf_base + conf + r * 0xBB67AE85
    uint32_t rk0[10], rk1[10];
    int lat0;                // lattice handled by blockIdx.x == 0
    int use_override;        // 1: beta_override / sweep_override instead of ladder / cycle
    double beta_override;
    uint32_t sweep_override;
    int* flips;              // accepted flips per site, row (conf * nrep + slot) of lat_stride
                             // ints (nullptr: not counted; generic kernels only)
    int* err;                // set to 1 when a bounded wait of a kernel gave up (or nullptr)
    int uf_tries;            // union-find attempts per bond before the labelling gives up
    int pdl;                 // host side: the launch may overlap the stream's previous kernel
    int zero_obs;            // generic global-memory sweep: this launch zeroes its lattices'
                             // observables (the first colour phase of a cycle)
                             // (programmatic dependent launch; global-memory kernels only)
    int slot0, nslots;       // HBM sweep kernel: temperature slots [slot0, slot0 + nslots) of
                             // every configuration of the launch, each slot's lattice found
                             // through rep_at_temp (nslots = 0: lattices lat0 .. in order)
};

// Replica-indexed arrays are laid out conf by conf: conf c owns entries rbase[c] ..
// rbase[c] + nreps[c] - 1 (replica, slot or pair index within the conf).
struct SwapArgs {
    const LatObs* obs;   // per replica
    const double* beta;  // per slot
    const int* nocc;     // per conf
    const int* rbase;    // per conf: first replica-indexed entry
    const int* nreps;    // per conf: ladder length
    int* rat;            // rep_at_temp, per slot
    int* tor;            // temp_of_rep, per replica
    double* sums;        // 22 per slot
    long long* nmeas;    // per slot
    long long* att;      // per pair
    long long* acc;      // per pair
    uint8_t* visited;    // per replica: bit0 cold end, bit1 hot end
    double* last_obs;    // 5 per replica
    uint32_t* ctl;       // ctl[0] cycle, ctl[1] swap phase (1 or 2), ctl[2] CTA ticket
    int nconf, measure;
    uint32_t seed, conf_base;
    // optional diagnostics of measured cycles
    int hist_bins;          // > 0: energy histogram per slot (counts, range set by 1st sample)
    long long* hist;        // [entries x hist_bins]
    double* hist_lo;        // per slot: lower edge (valid once hist_bs > 0)
    double* hist_bs;        // per slot: bin size, <= 0 until the first sample
    long long trace_cap;    // > 0: record the first trace_cap measured cycles
    int entries;            // replica-indexed entries of the context (trace row length)
    double* trace;          // [trace_cap x entries x 5] observables by slot
    int* trace_tor;         // [trace_cap x entries] temp_of_rep by replica
};

// Per-site accumulation of the replica at one temperature slot (Accumulate_local_nematic_average,
// J:1009-1025) for every conf of a group.
struct LocnemArgs {
    Geo g;
    const uint8_t* spins;    // group's first lattice
    long long lat_stride;
    const int* rat;          // rep_at_temp of the group's first entry
    int nrep, slot;
    int* loc_s;              // conf c at c * lat_stride (compact layout)
    int* loc_n;
    long long* samples;      // per conf of the group
};
cudaError_t launch_locnem(const LocnemArgs& a, int nconf, cudaStream_t st);

struct InitArgs {
    Geo g;
    uint8_t* spins;          // first lattice of the conf
    long long lat_stride;
    const uint8_t* occ;      // compact occupancy of the conf
    int nrep, start, axis;
    uint32_t seed, key1;
};

// Exact enumeration of a lattice of N <= 32 sites (enumerate.cu)
constexpr int kEnumBeta = 4;   // inverse temperatures per launch
constexpr int kEnumSums = 12;  // weighted sums per inverse temperature
struct EnumArgs {
    int N, LB;         // sites; low bits walked in Gray-code order by each thread
    double nocc, E0;   // occupied sites; lower bound of the energy
    double J1h, J1v, J2, J3;
    int nbeta;
    double beta[kEnumBeta];
    double p[32];
    int8_t nbr[32][10];  // reference neighbour slots m1..m10
    uint8_t occ[32], jh[32], jv[32], px[32], py[32];
};
int enum_blocks(const EnumArgs& a);
// message returned by j1j2c_last_error(NULL) (for entry points without a context)
void set_global_error(const char* msg);
cudaError_t launch_enumerate(const EnumArgs& a, double* partial, cudaStream_t st);

// Kernel variant of one sweep launch
struct SweepVariant {
    bool fp64;     // FP64 form (else FP32)
    bool quad;     // four sites per thread per colour phase (L % 8 == 0)
    bool stage_p;  // random field staged in shared memory
    bool masks;    // bond dilution present
    int mode;      // kModeSweep / kModeAudit
    int fixed_nt;  // > 0: shape-specialised kernel with this many threads per CTA
    bool stream;   // shape-specialised kernel: the streaming form
    int minb;      // shape-specialised kernel: resident CTAs per SM it is compiled for
    bool global;   // lattice in HBM, one launch per colour phase (too large for shared memory;
                   // with fixed_nt > 0 the shape-specialised form)
    bool vac;      // some conf has vacancies (shape-specialised kernels: vacancy handling on)
    int cluster;   // > 0: thread-block cluster of this many CTAs per lattice (distributed smem;
                   // quad: four sites per thread, else one)
    int rpt;       // shape-specialised HBM kernel: replicas per thread (1, 2 or 4)
    int rpc;       // shape-specialised shared-memory kernel: replicas per CTA (0 or 1: one)
    bool coop;     // global-memory form: every colour phase, sweep and the observables in one
                   // cooperative launch with grid barriers between the phases
    int threads;   // threads per CTA of the generic global-memory kernels (0: 256), of the
                   // cluster kernel (0: 512) and of the replicated-lattice cluster kernel
    int rep_cs;    // > 0: the lattice replicated in each of this many CTAs of a cluster, one site
                   // per thread (small batches)
};

// Global-memory path: one colour phase of sweep t of the cycle, and the observable reduction
// (adds into a.obs, which the caller zeroes first).
cudaError_t launch_sweep_global(const SweepArgs& a, const SweepVariant& v, int colour, int t,
                                int nlat, cudaStream_t st);
cudaError_t launch_measure_global(const SweepArgs& a, const SweepVariant& v, int nlat,
                                  cudaStream_t st);
// The cooperative form (v.coop): bar two zeroed words, a.obs of the lattices zeroed; with check,
// nothing is launched and the result says whether every CTA can be resident at once
cudaError_t launch_sweep_coop(const SweepArgs& a, const SweepVariant& v, int nlat, unsigned* bar,
                              cudaStream_t st, bool check);

// Cluster path: CTAs per lattice for a shape (0: not available), and the launch (PTSWAPEVER
// sweeps and the observables, added into a.obs, which the caller zeroes first).
int cluster_size_for(const Geo& g, bool fp64, bool masks, size_t max_smem);
int cluster_sizes(const Geo& g, bool fp64, bool masks, size_t max_smem, int* out, int cap);
// The replicated-lattice cluster form (v.rep_cs > 0): every sweep of the cycle and the
// observables (written, not added) in one launch; with check, nothing is launched and the result
// says whether such a cluster can be resident
cudaError_t launch_sweep_rep(const SweepArgs& a, const SweepVariant& v, int nlat,
                             cudaStream_t st, bool check);
size_t rep_smem_bytes(const Geo& g, bool fp64);  // its shared memory per CTA
cudaError_t launch_sweep_cluster(const SweepArgs& a, const SweepVariant& v, int nlat,
                                 cudaStream_t st);

// Shape-specialised kernels (sweep_fixed.cu): CTA sizes available for a shape, and the launch.
// A shape-specialised kernel: CTA size, field staged in shared memory, streaming form (one CTA
// per SM through a range of lattices, spins double-buffered by bulk copies)
struct FixedChoice {
    int nt;
    bool stage_p, stream;
    int minb;     // resident CTAs per SM the kernel is compiled for
    int rpc = 1;  // replicas of one configuration per CTA (their lattices share the field copy)
};
// int_cpl: J2 and J3 are integers with |J| <= 8 (SweepArgs::J2i, J3i); the FP32 kernels need it;
// nrep: ladder length (forms with several replicas per CTA need it to divide)
int fixed_candidates(bool fp64, int L, int H, bool masks, bool vac, bool int_cpl, int nrep,
                     FixedChoice* out, int cap);
// nlat lattices from a.lat0 (prepare: only set the kernel's shared-memory limit)
cudaError_t launch_fixed(const SweepArgs& a, bool fp64, bool vac, const FixedChoice& ch, int nlat,
                         size_t smem, cudaStream_t st, bool prepare);

// Shape-specialised kernels for lattices in HBM (one launch per colour phase): CTA size for a
// shape (0: none), and one colour phase (colour >= 0) or the observable reduction (colour < 0,
// added into a.obs, which the caller zeroes first).
// With rpt = 2 or 4 each thread updates its quad in that many replicas of one configuration
// (sharing the field loads); the launch falls back to 1 when the range is not whole
// configurations or rpt does not divide the replica count.
int fixed_hbm_threads(bool fp64, int L, int H, bool masks, bool int_cpl);
// CTA sizes of the shape's HBM kernels (the default first) into out; their number
int fixed_hbm_sizes(bool fp64, int L, int H, int* out, int cap);
cudaError_t launch_fixed_hbm(const SweepArgs& a, bool fp64, int nt, int colour, int t, int nlat,
                             int rpt, cudaStream_t st);

// One persistent launch over several lattice-shape groups (sweep_multi.cu).  A tile is R
// replicas of one configuration of a group; tile kinds exist for L = H = 16, 24, 32, 48.
struct GroupDesc {
    uint8_t* spins;           // the group's first lattice
    const float* pf;          // the group's first configuration's FP32 field
    long long lat_stride;     // bytes between lattices
    long long p_stride;       // elements between configurations' fields
    const double* beta;       // the group's first replica-indexed entry (by slot)
    const int* tor;           // temp_of_rep, same indexing
    LatObs* obs;              // observables of the group's first lattice
    int nrep, conf0;          // ladder length; the group's first configuration in the context
    int kind;                 // tile kind (multi_tile_kind)
};
struct MultiArgs {
    SweepArgs a;              // couplings, cycle counter, sweeps, key schedule of the context's
                              // conf_base (a tile passes conf0 + its configuration)
    const GroupDesc* groups;  // device array
    const int2* tasks;        // (group, first lattice of the tile), largest tiles first
    int ntasks;
    unsigned* queue;          // [0]: next task, zero at each launch
};
int multi_tile_kind(int L, int H);   // -1: the shape has no tile
int multi_tile_lattices(int kind);   // replicas of one configuration per tile
size_t multi_smem_bytes();           // dynamic shared memory of the launch (its largest tile)
int multi_threads();                 // threads per CTA
// grid: CTAs (at most one per SM); prepare: only raise the shared-memory limit
cudaError_t launch_multi(const MultiArgs& m, bool vac, int grid, cudaStream_t st, bool prepare);

size_t sweep_smem_bytes(const Geo& g, const SweepVariant& v);
cudaError_t prepare_sweep_variant(const SweepVariant& v, size_t smem);
cudaError_t launch_sweep(const SweepArgs& a, const SweepVariant& v, int nblocks, int nthreads,
                         size_t smem, cudaStream_t st);
cudaError_t launch_swap(const SwapArgs& a, cudaStream_t st, bool pdl = false);
// Wolff forms: seed-cluster growth (default), slab union-find labelling in shared memory,
// per-site union-find labelling in global memory; all three flip the same cluster.
enum WolffForm { kWolffGrow = 0, kWolffSlab = 1, kWolffSite = 2 };
// grow_cs: CTAs per lattice of the growth form (1, 2 or 4: a thread-block cluster)
cudaError_t launch_wolff(const SweepArgs& a, bool fp64, bool masks, int nlat, int* labels,
                         long long lab_stride, long long* csize, int* err, cudaStream_t st,
                         WolffForm form, int grow_cs);
int wolff_grow_clusters(bool fp64, bool masks, int cs);  // resident clusters of cs CTAs
// The growth form for the lattices at temperature slots [slot0, slot0 + nslots) of the group's
// nconf configurations (a.nrep slots each), cs CTAs per lattice; with act (one byte per site,
// lattice l at act + l * act_stride, filled by launch_wolff_bits for the same lattices and cycle)
// the bonds' activation is read from it (one CTA per lattice)
cudaError_t launch_wolff_grow(const SweepArgs& a, bool fp64, bool masks, int nconf, int slot0,
                              int nslots, int cs, int* labels, long long lab_stride,
                              long long* csize, cudaStream_t st, const uint8_t* act = nullptr,
                              long long act_stride = 0);
// The activation of every owned bond of the lattices at slots [slot0, slot0 + nslots) for the
// next growth of the same cycle, exactly as the growth form would decide it
cudaError_t launch_wolff_bits(const SweepArgs& a, bool fp64, bool masks, int nconf, int slot0,
                              int nslots, uint8_t* act, long long act_stride, cudaStream_t st);
int wolff_slab_planes(const Geo& g);  // planes per shared-memory slab of the Wolff labelling
cudaError_t launch_init(const InitArgs& a, cudaStream_t st);

}  // namespace j1j2
