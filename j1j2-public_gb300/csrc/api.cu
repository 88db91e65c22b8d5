// C-ABI of libj1j2cuda: context management, layout conversion between the reference's site order
// and the engine's colour-compact layout, the CUDA-graph replay of one PT cycle, and the outputs.
//
// A context holds one or more lattice-shape groups (mixed L in one batch).  Each group has its
// own kernel variant; one PT cycle is one graph: the groups' sweep launches as parallel branches,
// then one swap / accumulate launch over every conf.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/j1j2c.h"
#include "engine.h"

using namespace j1j2;

namespace {

thread_local std::string g_create_error;

}  // namespace

void j1j2::set_global_error(const char* msg) { g_create_error = msg; }

namespace {

// Temperature ranges of the split Wolff + sweep cycle at most (one stream each)
constexpr int kSplitRanges = 8;

struct Group {
    Geo g{};
    int nconf = 0, nrep = 0, conf0 = 0, rep0 = 0, block_threads = 0;
    long long lat_stride = 0, p_stride = 0;        // bytes per lattice, field elements per conf
    long long spin_off = 0, p_off = 0, mask_off = 0;  // offsets into the context's arrays
    long long lab_off = 0;                            // offset into the Wolff label scratch
    SweepVariant var{};
    int nthreads = 0;
    size_t smem = 0;
    bool tuned = false;
    int wolff_cs = 0;  // CTAs per lattice of the Wolff growth kernel (0: not tuned, 1)
    int wolff_k = 0;   // 0 < k < nrep: only the k coldest slots take wolff_cs CTAs, the rest one
    // HBM sweep form with Wolff: 0 < split[0] < nrep runs the Wolff update, sweeps and
    // observables of every configuration's temperature slots as up to kSplitRanges ranges on as
    // many streams, the boundaries 0 < split[0] < split[1] < ... < nrep (a 0 ends the list);
    // the coldest range takes split_cs CTAs per growing cluster
    int split[kSplitRanges - 1] = {};
    int split_cs = 1;
    // the Wolff update of the cold slots (split form: slots [0, split[0]); unsplit: every slot)
    // reads bond activations decided beforehand on every SM (wolff_bits_kernel)
    bool split_bits = false;
    int nlat() const { return nconf * nrep; }
};

constexpr int kProfPool = 64;  // profiling event pairs in flight before the host reads them

struct Ctx {
    j1j2c_params P{};
    std::vector<Group> G;
    int nconf = 0, nentries = 0;  // confs, replica-indexed entries (sum of nconf*nrep)
    std::vector<int> conf_group, conf_rbase, conf_nrep;

    uint8_t* d_spins = nullptr;
    float* d_pf = nullptr;
    double* d_pd = nullptr;
    uint8_t* d_bm = nullptr;
    uint8_t* d_occ = nullptr;
    double* d_beta = nullptr;
    float* d_kb = nullptr;  // by slot: the FP32 acceptance scale of each beta
    int* d_rat = nullptr;
    int* d_tor = nullptr;
    LatObs* d_obs = nullptr;
    double* d_sums = nullptr;
    long long* d_nmeas = nullptr;
    long long* d_att = nullptr;
    long long* d_acc = nullptr;
    uint8_t* d_vis = nullptr;
    double* d_last = nullptr;
    uint32_t* d_ctl = nullptr;
    int* d_nocc = nullptr;
    int* d_rbase = nullptr;
    int* d_nreps = nullptr;
    unsigned long long* d_audit = nullptr;
    int* d_labels = nullptr;        // Wolff union-find labels / cluster list, one int per site
    uint8_t* d_act = nullptr;       // Wolff bond activation bits, one byte per site (first use)
    long long* d_csize = nullptr;   // Wolff cluster size of the last update, per replica
    int* d_err = nullptr;           // device error word (union-find retry overflow)
    unsigned* d_gbar = nullptr;     // grid-barrier words of the cooperative form, two per group
    int uf_tries = 1 << 20;         // union-find attempts per bond (j1j2c_set_retry_budget)
    long long lab_ints = 0;
    bool wolff = false;

    std::vector<uint8_t> have_dis, have_ladder, have_spins;
    std::vector<int> nocc, conf_masks, conf_vac;
    bool masks = false, vac = false;

    cudaStream_t own = nullptr, st = nullptr;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> join_ev;
    cudaEvent_t fork_ev = nullptr;
    // per group: the fork event, and kSplitRanges - 1 side streams with their join events, of
    // a Wolff update split over two launches or of the split Wolff + sweep cycle
    std::vector<cudaStream_t> wside;
    std::vector<cudaEvent_t> wfork, wjoin;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaGraph_t graph_src[2] = {nullptr, nullptr};  // kept: its event-record nodes are retargeted
    cudaGraphNode_t graph_ev[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    long long occ_total = 0;

    // J1J2C_FLAG_PROFILE: every cycle brackets its sweep launches with its own pair of a pool of
    // event pairs (the graph's event-record nodes retargeted before each launch); the pairs are
    // read after the run's final synchronisation, so profiling adds no host wait between cycles
    bool profile = false;
    // several lattice-shape groups swept by one persistent launch (sweep_multi.cu) instead of one
    // graph branch per group: chosen at the first run (multi_tuned), its device tables on first use
    bool multi = false, multi_tuned = false;
    GroupDesc* d_gdesc = nullptr;
    int2* d_tasks = nullptr;
    unsigned* d_queue = nullptr;
    int ntasks = 0, multi_grid = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> pev0, pev1;
    int prof_pending = 0;
    double prof_ms = 0.0;
    long long prof_launches = 0, prof_attempts = 0;

    // optional diagnostics (j1j2c_set_diagnostics)
    j1j2c_diagnostics diag{-1, 0, 0, 0};
    long long spin_bytes = 0, mask_bytes = 0, p_elems = 0;
    int* d_loc_s = nullptr;             // per-site sums of s (conf at mask offsets)
    int* d_loc_n = nullptr;             // per-site sums of the local nematic term
    long long* d_loc_samples = nullptr; // per conf
    long long* d_hist = nullptr;        // [entries x bins]
    double* d_hist_lo = nullptr;
    double* d_hist_bs = nullptr;
    double* d_trace = nullptr;          // [cycles x entries x 5]
    int* d_trace_tor = nullptr;         // [cycles x entries]
    int* d_flips = nullptr;             // flip counts, laid out like the spins

    uint32_t host_ctl[4] = {0, 1, 0, 0};
    std::string err;
};

int fail(Ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

int cuda_fail(Ctx* c, cudaError_t e, const char* what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(c, e == cudaErrorMemoryAllocation ? J1J2C_ENOMEM : J1J2C_ECUDA, m);
}

#define CK(c, call)                                               \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail((c), e_, #call); \
    } while (0)

// j1j2c_inject_fault: a one-shot failure of the next device allocation (1) or the next PT-cycle
// launch (2) that any context of the process makes; the failure is reported as CUDA would report
// it, without calling CUDA, so the device and its context are untouched
std::atomic<int> g_inject{0};

bool take_injected(int kind)
{
    int k = kind;
    return g_inject.load() == kind && g_inject.compare_exchange_strong(k, 0);
}

// every device allocation of the engine comes through here
cudaError_t dev_malloc(void** p, size_t bytes)
{
    if (take_injected(1)) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

template <class T>
cudaError_t dev_malloc(T** p, size_t bytes)
{
    return dev_malloc(reinterpret_cast<void**>(p), bytes);
}

template <class T>
cudaError_t dalloc(T** p, size_t n)
{
    return dev_malloc(reinterpret_cast<void**>(p), n * sizeof(T) + 16);
}

// The Wolff label scratch and growth list (one int per site of every lattice), filled with
// empty list entries (all bits set): the growth kernels leave every position they used empty
// again, and the level-free growth reads an entry as present once it is not empty
cudaError_t fill_labels(Ctx* c)
{
    const cudaError_t e =
        cudaMemsetAsync(c->d_labels, 0xFF, sizeof(int) * (size_t)c->lab_ints, c->own);
    return e == cudaSuccess ? cudaStreamSynchronize(c->own) : e;
}

cudaError_t alloc_labels(Ctx* c)
{
    if (c->d_labels) return cudaSuccess;
    const cudaError_t e = dalloc(&c->d_labels, (size_t)c->lab_ints);
    return e == cudaSuccess ? fill_labels(c) : e;
}

void free_graphs(Ctx* c)
{
    for (int m = 0; m < 2; ++m) {
        if (c->graph[m]) cudaGraphExecDestroy(c->graph[m]);
        if (c->graph_src[m]) cudaGraphDestroy(c->graph_src[m]);
        c->graph[m] = nullptr;
        c->graph_src[m] = nullptr;
        c->graph_ev[m][0] = c->graph_ev[m][1] = nullptr;
    }
}

void release(Ctx* c)
{
    free_graphs(c);
    void* ptrs[] = {c->d_spins, c->d_pf,    c->d_pd,   c->d_bm,    c->d_occ,   c->d_beta,
                    c->d_kb,
                    c->d_rat,   c->d_tor,   c->d_obs,  c->d_sums,  c->d_nmeas, c->d_att,
                    c->d_acc,   c->d_vis,   c->d_last, c->d_ctl,   c->d_nocc,  c->d_rbase,
                    c->d_nreps, c->d_audit, c->d_labels, c->d_act, c->d_csize, c->d_err,
                    c->d_loc_s, c->d_loc_n, c->d_loc_samples, c->d_hist, c->d_hist_lo,
                    c->d_hist_bs, c->d_trace, c->d_trace_tor, c->d_flips, c->d_gdesc,
                    c->d_tasks, c->d_queue, c->d_gbar};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (auto s : c->side) cudaStreamDestroy(s);
    for (auto e : c->join_ev) cudaEventDestroy(e);
    for (auto s : c->wside)
        if (s) cudaStreamDestroy(s);
    for (auto e : c->wfork)
        if (e) cudaEventDestroy(e);
    for (auto e : c->wjoin)
        if (e) cudaEventDestroy(e);
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (auto e : c->pev0) cudaEventDestroy(e);
    for (auto e : c->pev1) cudaEventDestroy(e);
    if (c->own) cudaStreamDestroy(c->own);
}

// Shared memory of a cluster-path CTA that still lets two CTAs share an SM
constexpr size_t kClusterCtaSmem = 112 * 1024;

size_t smem_budget(Ctx* c)
{
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->P.device) !=
        cudaSuccess)
        return 0;
    return (size_t)optin - 2048;  // static shared memory of the reduction
}

// threads of a per-site cluster CTA: its sites of one colour, in whole warps, at most 512
int cluster_site_threads(const Group& grp, int cs)
{
    int nt = ((grp.g.Nc / cs + 31) / 32) * 32;
    return nt > 512 ? 512 : nt;
}

// J2 and J3 are integers with |J| <= 8 in FP32, as the FP32 shape-specialised kernels need (their
// first two field terms are then formed exactly in integer arithmetic)
bool int_couplings(const Ctx* c)
{
    const float j2 = (float)c->P.J2, j3 = (float)c->P.J3;
    return std::fabs(j2) <= 8.0f && std::fabs(j3) <= 8.0f && j2 == std::nearbyint(j2) &&
           j3 == std::nearbyint(j3);
}

// CTA size of the shape-specialised kernel for a group whose lattices stay in HBM (0: the
// generic global-memory kernel).  Like the shared-memory ones it counts no flips and handles no
// bond dilution; the test flags GENERIC and NO_FIXED pin the generic kernel.
int hbm_fixed_threads(const Ctx* c, const Group& grp, bool fp64)
{
    if ((c->P.flags & (J1J2C_FLAG_GENERIC | J1J2C_FLAG_NO_FIXED)) || c->diag.flip_counts)
        return 0;
    return fixed_hbm_threads(fp64, grp.g.L, grp.g.H, c->masks, int_couplings(c));
}

// Kernel shape for a group: the shape-specialised kernel when one exists for (precision, L, H)
// and no bond is diluted (its CTA size autotuned at the first run unless block_threads names
// one); else the generic CTA-per-lattice kernel with the lattice in shared memory (quad path when
// L/2 is a multiple of 4, else per-site; the field staged when it fits); else, for lattices too
// large for shared memory, the global-memory path with one launch per colour phase.
int choose_variant(Ctx* c, Group& grp, bool fp64, SweepVariant& v, size_t& smem, int& nthreads)
{
    const size_t budget = smem_budget(c);
    if (budget == 0) return fail(c, J1J2C_ECUDA, "cannot query the shared-memory limit");
    const uint32_t fl = c->P.flags;
    v = SweepVariant{};
    v.fp64 = fp64;
    v.masks = c->masks;
    v.vac = c->vac;
    v.mode = kModeSweep;
    const bool quad_ok = (grp.g.Lh % 4 == 0) && !(fl & J1J2C_FLAG_GENERIC);
    if ((fl & J1J2C_FLAG_CLUSTER) && grp.g.Lh % 4 == 0) {
        // the largest cluster; with the GENERIC flag one site per thread
        int cs[16];
        const int n = cluster_sizes(grp.g, fp64, c->masks, budget, cs, 16);
        if (n > 0) {
            v.quad = quad_ok;
            v.cluster = cs[n - 1];
            v.stage_p = false;
            smem = (size_t)grp.g.N / (size_t)cs[n - 1];
            nthreads = quad_ok ? 512 : cluster_site_threads(grp, cs[n - 1]);
            v.threads = nthreads;
            return J1J2C_OK;
        }
    }
    // the shape-specialised kernels do not count flips
    if (!(fl & (J1J2C_FLAG_GENERIC | J1J2C_FLAG_NO_FIXED | J1J2C_FLAG_GLOBAL)) &&
        !c->diag.flip_counts) {
        FixedChoice fc[16];
        const int n = fixed_candidates(fp64, grp.g.L, grp.g.H, c->masks, c->vac,
                                       int_couplings(c), grp.nrep, fc, 16);
        // the first one-replica-per-CTA form (or the block_threads one); the streaming form or
        // two replicas per CTA when a test flag asks for it
        const bool stream = (fl & J1J2C_FLAG_STREAM) != 0;
        const int rpc = (fl & J1J2C_FLAG_PAIRS) ? 2 : 1;
        int pick = -1;
        for (int k = n - 1; k >= 0; --k)
            if (fc[k].stream == stream && fc[k].rpc == rpc &&
                (grp.block_threads == 0 || fc[k].nt == grp.block_threads))
                pick = k;
        if (pick >= 0) {
            v.fixed_nt = fc[pick].nt;
            v.quad = true;
            v.stage_p = fc[pick].stage_p;
            v.stream = fc[pick].stream;
            v.minb = fc[pick].minb;
            v.rpc = fc[pick].rpc;
            smem = sweep_smem_bytes(grp.g, v);
            if (smem <= budget) {
                nthreads = fc[pick].nt;
                SweepArgs none{};
                none.g = grp.g;
                CK(c, launch_fixed(none, fp64, c->vac, fc[pick], 0, smem, nullptr, true));
                return J1J2C_OK;
            }
            v.fixed_nt = 0;
            v.stream = false;
        }
    }
    v.quad = quad_ok;
    const int work = v.quad ? grp.g.Nc / 4 : grp.g.Nc;
    v.stage_p = true;
    smem = sweep_smem_bytes(grp.g, v);
    if (smem > budget) {
        v.stage_p = false;
        smem = sweep_smem_bytes(grp.g, v);
    }
    if (smem > budget && !(fl & J1J2C_FLAG_GLOBAL) && v.quad) {
        // the lattice in the distributed shared memory of a thread-block cluster: prefer CTAs
        // small enough for two per SM
        int cs = cluster_size_for(grp.g, fp64, c->masks, kClusterCtaSmem);
        if (cs == 0) cs = cluster_size_for(grp.g, fp64, c->masks, budget);
        if (cs > 0) {
            v.cluster = cs;
            v.stage_p = false;
            smem = (size_t)grp.g.N / (size_t)cs;
            nthreads = 512;
            return J1J2C_OK;
        }
    }
    if (smem > budget || (fl & J1J2C_FLAG_GLOBAL)) {
        v.global = true;
        v.stage_p = false;
        v.fixed_nt = hbm_fixed_threads(c, grp, fp64);
        if (v.fixed_nt > 0 && grp.block_threads > 0) {  // one of the HBM kernel's CTA sizes
            int sz[4];
            const int n = fixed_hbm_sizes(fp64, grp.g.L, grp.g.H, sz, 4);
            for (int k = 0; k < n; ++k)
                if (sz[k] == grp.block_threads) v.fixed_nt = sz[k];
        }
        v.rpt = grp.nrep % 4 == 0 ? 4 : grp.nrep % 2 == 0 ? 2 : 1;
        smem = 0;
        nthreads = v.fixed_nt > 0 ? v.fixed_nt : 256;
        return J1J2C_OK;
    }
    if (grp.block_threads > 0) {
        nthreads = grp.block_threads;
    } else {
        nthreads = ((work + 31) / 32) * 32;
        if (nthreads > 1024) nthreads = 1024;
        if (nthreads < 64) nthreads = 64;
    }
    CK(c, prepare_sweep_variant(v, smem));
    return J1J2C_OK;
}

SweepArgs group_args(Ctx* c, const Group& grp)
{
    SweepArgs a{};
    a.g = grp.g;
    a.spins = c->d_spins + grp.spin_off;
    a.lat_stride = grp.lat_stride;
    a.pf = c->d_pf + grp.p_off;
    a.pd = c->d_pd + grp.p_off;
    a.bm = c->masks ? c->d_bm + grp.mask_off : nullptr;
    a.p_stride = grp.p_stride;
    a.beta = c->d_beta + grp.rep0;
    a.kb = c->d_kb + grp.rep0;
    a.temp_of_rep = c->d_tor + grp.rep0;
    a.rep_at_temp = c->d_rat + grp.rep0;
    a.ctl = c->d_ctl;
    a.obs = c->d_obs + grp.rep0;
    a.audit = c->d_audit;
    a.J1h = c->P.J1h;
    a.J1v = c->P.J1v;
    a.J2 = c->P.J2;
    a.J3 = c->P.J3;
    a.J1hf = (float)c->P.J1h;
    a.J1vf = (float)c->P.J1v;
    a.J2f = (float)c->P.J2;
    a.J3f = (float)c->P.J3;
    if (int_couplings(c)) {
        a.J2i = (int)a.J2f;
        a.J3i = (int)a.J3f;
        const int bias = 4 * std::abs(a.J3i) + 8 * std::abs(a.J2i);
        a.ij_bias = 0x01010101u * (uint32_t)bias;
        a.ij_off = 8388608.0f + (float)(bias + 2 * a.J3i + 4 * a.J2i);
    }
    a.nrep = grp.nrep;
    a.nsweeps = c->P.ptswapever;
    a.ptswapever = c->P.ptswapever;
    a.seed = c->P.seed;
    a.conf_base = c->P.conf_base + (uint32_t)grp.conf0;
    for (int r = 0; r < 10; ++r) {
        a.rk0[r] = a.seed + (uint32_t)r * 0x9E3779B9u;
        a.rk1[r] = a.conf_base + (uint32_t)r * 0xBB67AE85u;
    }
    a.lat0 = 0;
    a.use_override = 0;
    a.flips = c->d_flips ? c->d_flips + grp.spin_off : nullptr;
    a.err = c->d_err;
    a.uf_tries = c->uf_tries;
    return a;
}

SwapArgs swap_args(Ctx* c, int measure)
{
    SwapArgs s{};
    s.obs = c->d_obs;
    s.beta = c->d_beta;
    s.nocc = c->d_nocc;
    s.rbase = c->d_rbase;
    s.nreps = c->d_nreps;
    s.rat = c->d_rat;
    s.tor = c->d_tor;
    s.sums = c->d_sums;
    s.nmeas = c->d_nmeas;
    s.att = c->d_att;
    s.acc = c->d_acc;
    s.visited = c->d_vis;
    s.last_obs = c->d_last;
    s.ctl = c->d_ctl;
    s.nconf = c->nconf;
    s.measure = measure;
    s.seed = c->P.seed;
    s.conf_base = c->P.conf_base;
    s.hist_bins = c->d_hist ? c->diag.hist_bins : 0;
    s.hist = c->d_hist;
    s.hist_lo = c->d_hist_lo;
    s.hist_bs = c->d_hist_bs;
    s.trace_cap = c->d_trace ? c->diag.trace_cycles : 0;
    s.entries = c->nentries;
    s.trace = c->d_trace;
    s.trace_tor = c->d_trace_tor;
    return s;
}

// Accumulate_local_nematic_average of every conf whose ladder has the diagnostic slot
cudaError_t enqueue_locnem(Ctx* c, cudaStream_t st)
{
    for (const Group& grp : c->G) {
        if (c->diag.locnem_slot >= grp.nrep) continue;
        LocnemArgs a{};
        a.g = grp.g;
        a.spins = c->d_spins + grp.spin_off;
        a.lat_stride = grp.lat_stride;
        a.rat = c->d_rat + grp.rep0;
        a.nrep = grp.nrep;
        a.slot = c->diag.locnem_slot;
        a.loc_s = c->d_loc_s + grp.mask_off;
        a.loc_n = c->d_loc_n + grp.mask_off;
        a.samples = c->d_loc_samples + grp.conf0;
        cudaError_t e = launch_locnem(a, grp.nconf, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// CTAs per lattice of the Wolff growth kernel: pinned by the test flags (both: 2 CTAs for the
// coldest quarter of the slots, one for the rest), else the tuned count
constexpr uint32_t kWolffPinned = J1J2C_FLAG_WOLFF_CS2 | J1J2C_FLAG_WOLFF_CS4;

int wolff_cs_of(const Ctx* c, const Group& grp)
{
    const uint32_t f = c->P.flags & kWolffPinned;
    if (f == kWolffPinned || f == J1J2C_FLAG_WOLFF_CS2) return 2;
    if (f == J1J2C_FLAG_WOLFF_CS4) return 4;
    return grp.wolff_cs > 0 ? grp.wolff_cs : 1;
}

// CTAs-per-lattice argument of a growth launch: one-CTA growths in the level-free form (-1)
// where J1J2C_FLAG_WOLFF_ASYNC pins it
int grow_cs(const Ctx* c, const Group& grp, int cs)
{
    (void)grp;
    return cs == 1 && (c->P.flags & J1J2C_FLAG_WOLFF_ASYNC) ? -1 : cs;
}

// Coldest slots that take wolff_cs_of CTAs (0: every slot)
int wolff_k_of(const Ctx* c, const Group& grp)
{
    const uint32_t f = c->P.flags & kWolffPinned;
    if (f == kWolffPinned) return grp.nrep >= 2 ? (grp.nrep / 4 > 0 ? grp.nrep / 4 : 1) : 0;
    return f ? 0 : grp.wolff_k;
}

// The group's Wolff side streams and events (created with the context)
cudaError_t wolff_side(Ctx* c, const Group& grp)
{
    constexpr size_t ns = kSplitRanges - 1;
    const size_t k = (size_t)(&grp - c->G.data());
    if (c->wfork.size() < c->G.size()) {
        c->wside.resize(c->G.size() * ns, nullptr);
        c->wjoin.resize(c->G.size() * ns, nullptr);
        c->wfork.resize(c->G.size(), nullptr);
    }
    cudaError_t e = cudaSuccess;
    for (size_t j = k * ns; j < (k + 1) * ns && e == cudaSuccess; ++j) {
        if (!c->wside[j]) e = cudaStreamCreateWithFlags(&c->wside[j], cudaStreamNonBlocking);
        if (e == cudaSuccess && !c->wjoin[j])
            e = cudaEventCreateWithFlags(&c->wjoin[j], cudaEventDisableTiming);
    }
    if (e == cudaSuccess && !c->wfork[k])
        e = cudaEventCreateWithFlags(&c->wfork[k], cudaEventDisableTiming);
    return e;
}

// Side stream j (0 .. kSplitRanges - 2) of group gi, and its join event
cudaStream_t side_of(const Ctx* c, size_t gi, int j)
{
    return c->wside[gi * (kSplitRanges - 1) + (size_t)j];
}
cudaEvent_t join_of(const Ctx* c, size_t gi, int j)
{
    return c->wjoin[gi * (kSplitRanges - 1) + (size_t)j];
}

// The growth reads bond activations decided beforehand (test flag, or the split tuner's choice)
bool bits_of(const Ctx* c, const Group& grp)
{
    return (c->P.flags & J1J2C_FLAG_WOLFF_BITS) != 0 || grp.split_bits;
}

// Device buffer of the activation bits (the spins' layout, one byte per site), on first use
int ensure_act(Ctx* c)
{
    if (!c->d_act) CK(c, dalloc(&c->d_act, (size_t)c->spin_bytes));
    return J1J2C_OK;
}

// Growth form over the group's lattices with a (spins of) a: the k coldest slots of every
// configuration with cs CTAs per lattice and the other slots with one, as two concurrent
// launches (0 < k < nrep), else every lattice with cs CTAs.  With bond activations decided
// beforehand (bits_of; c->d_act allocated): every lattice, one CTA each, reading them.
cudaError_t enqueue_wolff_grow(Ctx* c, const Group& grp, const SweepArgs& a, int cs, int k,
                               cudaStream_t st)
{
    int* lab = c->d_labels + grp.lab_off;
    long long* cz = c->d_csize + grp.rep0;
    if (bits_of(c, grp) && c->d_act) {
        uint8_t* act = c->d_act + grp.spin_off;
        cudaError_t e = launch_wolff_bits(a, grp.var.fp64, c->masks, grp.nconf, 0, grp.nrep, act,
                                          grp.lat_stride, st);
        if (e != cudaSuccess) return e;
        return launch_wolff_grow(a, grp.var.fp64, c->masks, grp.nconf, 0, grp.nrep, 1, lab,
                                 grp.lat_stride, cz, st, act, grp.lat_stride);
    }
    if (k <= 0 || k >= grp.nrep || cs == 1)
        return launch_wolff_grow(a, grp.var.fp64, c->masks, grp.nconf, 0, grp.nrep,
                                 grow_cs(c, grp, cs), lab, grp.lat_stride, cz, st);
    const size_t gi = (size_t)(&grp - c->G.data());
    cudaError_t e;
    const cudaStream_t side = side_of(c, gi, 0);
    if ((e = cudaEventRecord(c->wfork[gi], st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(side, c->wfork[gi], 0)) != cudaSuccess) return e;
    if ((e = launch_wolff_grow(a, grp.var.fp64, c->masks, grp.nconf, 0, k, cs, lab,
                               grp.lat_stride, cz, st)) != cudaSuccess)
        return e;
    if ((e = launch_wolff_grow(a, grp.var.fp64, c->masks, grp.nconf, k, grp.nrep - k,
                               grow_cs(c, grp, 1), lab, grp.lat_stride, cz, side)) !=
        cudaSuccess)
        return e;
    if ((e = cudaEventRecord(join_of(c, gi, 0), side)) != cudaSuccess) return e;
    return cudaStreamWaitEvent(st, join_of(c, gi, 0), 0);
}

// The split points of the split Wolff + sweep form into pts (kSplitRanges - 1 entries, a 0
// ending the list; pts[0] = 0: not split).  J1J2C_FLAG_WOLFF_SPLIT pins them: a quarter of the
// slots, or J1J2C_SPLIT="k1,k2,..." from the environment (tests); else the tuner's choice.
void split_of(const Ctx* c, const Group& grp, int* pts)
{
    for (int j = 0; j < kSplitRanges - 1; ++j) pts[j] = 0;
    if (!c->wolff || !grp.var.global || grp.var.fixed_nt <= 0) return;
    if (!(c->P.flags & J1J2C_FLAG_WOLFF_SPLIT)) {
        for (int j = 0; j < kSplitRanges - 1; ++j) pts[j] = grp.split[j];
        return;
    }
    pts[0] = grp.nrep >= 2 ? (grp.nrep + 3) / 4 : 0;
    const char* env = std::getenv("J1J2C_SPLIT");
    // the ascending prefix inside (0, nrep) of the comma-separated list
    for (int j = 0, prev = 0; env && *env && j < kSplitRanges - 1; ++j) {
        char* end = nullptr;
        const long x = std::strtol(env, &end, 10);
        if (end == env || x <= prev || x >= grp.nrep) break;
        pts[j] = prev = (int)x;
        env = *end == ',' ? end + 1 : end;
    }
}

// CTAs per growing cluster of the split form's cold slots
int split_cs_of(const Ctx* c, const Group& grp)
{
    if (c->P.flags & J1J2C_FLAG_WOLFF_SPLIT) return wolff_cs_of(c, grp);
    return grp.split_cs;
}

// The Wolff update, PTSWAPEVER sweeps and the observables of a group in the HBM sweep form (a:
// its arguments, whole configurations), split by temperature slot at the points pts (ascending,
// a 0 ending the list): the coldest range of every configuration on stream st, each other
// range on one of the group's side streams.  The hotter lattices' sweeps run while the colder
// lattices' clusters still grow, and a short coldest range keeps the sweeps that follow the
// longest growths short; every lattice keeps its own order (its Wolff update, then its sweeps,
// then its observables).
cudaError_t enqueue_split(Ctx* c, const Group& grp, const SweepVariant& v, SweepArgs a,
                          const int* pts, int cs, cudaStream_t st, bool bits)
{
    const size_t gi = (size_t)(&grp - c->G.data());
    const int nlat = grp.nlat();
    int* lab = c->d_labels + grp.lab_off;
    long long* cz = c->d_csize + grp.rep0;
    cudaError_t e;
    if ((e = cudaMemsetAsync(cz, 0, sizeof(long long) * nlat, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(a.obs + a.lat0, 0, sizeof(LatObs) * nlat, st)) != cudaSuccess)
        return e;
    int s0[kSplitRanges] = {0}, nh = 1;  // range h: slots [s0[h], s0[h + 1])
    while (nh < kSplitRanges && pts[nh - 1] > s0[nh - 1] && pts[nh - 1] < grp.nrep) {
        s0[nh] = pts[nh - 1];
        ++nh;
    }
    if (nh < 2) return cudaErrorInvalidValue;
    const int k = s0[1];
    if ((e = cudaEventRecord(c->wfork[gi], st)) != cudaSuccess) return e;
    cudaStream_t ss[kSplitRanges] = {st};
    for (int h = 1; h < nh; ++h) {
        ss[h] = side_of(c, gi, h - 1);
        if ((e = cudaStreamWaitEvent(ss[h], c->wfork[gi], 0)) != cudaSuccess) return e;
    }
    for (int h = 0; h < nh; ++h) {
        const int ns = (h + 1 < nh ? s0[h + 1] : grp.nrep) - s0[h];
        SweepArgs b = a;
        if (h == 0 && bits && c->d_act) {  // the cold slots: activations first, on every SM
            uint8_t* act = c->d_act + grp.spin_off;
            if ((e = launch_wolff_bits(b, v.fp64, c->masks, grp.nconf, 0, k, act, grp.lat_stride,
                                       st)) != cudaSuccess)
                return e;
            e = launch_wolff_grow(b, v.fp64, c->masks, grp.nconf, 0, k, 1, lab, grp.lat_stride,
                                  cz, st, act, grp.lat_stride);
        } else {
            e = launch_wolff_grow(b, v.fp64, c->masks, grp.nconf, s0[h], ns,
                                  grow_cs(c, grp, h == 0 ? cs : 1), lab, grp.lat_stride, cz,
                                  ss[h]);
        }
        if (e != cudaSuccess) return e;
        b.slot0 = s0[h];
        b.nslots = ns;
        for (int t = 0; t < a.nsweeps; ++t)
            for (int col = 0; col < 8; ++col) {
                b.pdl = (t > 0 || col > 0) ? 1 : 0;
                if ((e = launch_sweep_global(b, v, col, t, nlat, ss[h])) != cudaSuccess) return e;
            }
        // each range measures its own lattices, so a hotter range's measurement overlaps the
        // colder ranges' sweeps
        b.pdl = 1;
        if ((e = launch_measure_global(b, v, nlat, ss[h])) != cudaSuccess) return e;
    }
    for (int h = 1; h < nh; ++h) {
        if ((e = cudaEventRecord(join_of(c, gi, h - 1), ss[h])) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(st, join_of(c, gi, h - 1), 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// PTSWAPEVER sweeps and the observable reduction of lattices [lat0, lat0 + nlat) of a group
cudaError_t enqueue_wolff(Ctx* c, const Group& grp, cudaStream_t st)
{
    SweepArgs a = group_args(c, grp);
    cudaError_t e = cudaMemsetAsync(c->d_csize + grp.rep0, 0, sizeof(long long) * grp.nlat(), st);
    if (e != cudaSuccess) return e;
    // default: seed-cluster growth; the labelling forms stay selectable for cross-checks
    const WolffForm form = (c->P.flags & J1J2C_FLAG_GENERIC)    ? kWolffSite
                           : (c->P.flags & J1J2C_FLAG_NO_FIXED) ? kWolffSlab
                                                                : kWolffGrow;
    const int cs = wolff_cs_of(c, grp);
    if (form == kWolffGrow) return enqueue_wolff_grow(c, grp, a, cs, wolff_k_of(c, grp), st);
    return launch_wolff(a, grp.var.fp64, c->masks, grp.nlat(), c->d_labels + grp.lab_off,
                        grp.lat_stride, c->d_csize + grp.rep0, c->d_err, st, form, cs);
}

cudaError_t enqueue_group(Ctx* c, const Group& grp, const SweepVariant& v, int nthreads,
                          size_t smem, SweepArgs a, int nlat, cudaStream_t st, bool cycle)
{
    cudaError_t e;
    if (cycle && c->wolff && nlat == grp.nlat() && v.global && v.fixed_nt > 0) {
        int pts[kSplitRanges - 1];
        split_of(c, grp, pts);
        if (pts[0] > 0)
            return enqueue_split(c, grp, v, a, pts, split_cs_of(c, grp), st, bits_of(c, grp));
    }
    if (cycle && c->wolff && (e = enqueue_wolff(c, grp, st)) != cudaSuccess) return e;
    if (v.rep_cs > 0) return launch_sweep_rep(a, v, nlat, st, false);  // writes the observables
    if (v.cluster > 0) {
        if ((e = cudaMemsetAsync(a.obs + a.lat0, 0, sizeof(LatObs) * nlat, st)) != cudaSuccess)
            return e;
        return launch_sweep_cluster(a, v, nlat, st);
    }
    if (!v.global) return launch_sweep(a, v, nlat, nthreads, smem, st);
    if (v.coop && c->d_gbar) {  // every phase in one cooperative launch
        const size_t gi = (size_t)(&grp - c->G.data());
        unsigned* bar = c->d_gbar + 2 * (gi < c->G.size() ? gi : 0);
        if ((e = cudaMemsetAsync(a.obs + a.lat0, 0, sizeof(LatObs) * nlat, st)) != cudaSuccess)
            return e;
        if ((e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st)) != cudaSuccess) return e;
        return launch_sweep_coop(a, v, nlat, bar, st, false);
    }
    // one launch per colour phase, every launch after the first following a kernel of the same
    // chain and overlapping its tail (programmatic dependent launch: each kernel waits for its
    // predecessor before any access).  The observables, which no sweep reads, are zeroed by the
    // first launch of the generic kernel (no graph node of its own) or before the chain.
    const bool zero_in_kernel = v.fixed_nt <= 0 && a.nsweeps > 0;
    if (!zero_in_kernel &&
        (e = cudaMemsetAsync(a.obs + a.lat0, 0, sizeof(LatObs) * nlat, st)) != cudaSuccess)
        return e;
    for (int t = 0; t < a.nsweeps; ++t)
        for (int col = 0; col < 8; ++col) {
            a.pdl = (t > 0 || col > 0) ? 1 : 0;
            a.zero_obs = zero_in_kernel && t == 0 && col == 0 ? 1 : 0;
            if ((e = launch_sweep_global(a, v, col, t, nlat, st)) != cudaSuccess) return e;
        }
    a.zero_obs = 0;
    a.pdl = 1;
    (void)grp;
    (void)c;
    return launch_measure_global(a, v, nlat, st);
}

// Every group of the context has a tile of the persistent multi-shape kernel: FP32 with integer
// J2, J3, no diluted bond, no flip counting, no test flag pinning another kernel, each shape one of
// L = H = 16, 24, 32, 48 with a ladder that the tile's replica count divides
bool multi_possible(Ctx* c)
{
    const uint32_t f = c->P.flags;
    if (c->G.size() < 2 || c->P.precision != J1J2C_FP32_BATCHED || c->masks ||
        !int_couplings(c) || c->diag.flip_counts ||
        (f & (J1J2C_FLAG_GENERIC | J1J2C_FLAG_NO_FIXED | J1J2C_FLAG_GLOBAL | J1J2C_FLAG_CLUSTER |
              J1J2C_FLAG_STREAM | J1J2C_FLAG_PAIRS)))
        return false;
    for (const Group& grp : c->G) {
        const int kind = multi_tile_kind(grp.g.L, grp.g.H);
        if (kind < 0 || grp.nrep % multi_tile_lattices(kind) != 0) return false;
    }
    return multi_smem_bytes() <= smem_budget(c);
}

// Every group's Wolff update (with J1J2C_FLAG_WOLFF), sweeps and observables of one PT cycle:
// one group on st; several as parallel graph branches on the side streams, joined on st; or
// (multi) the groups' Wolff updates on st, then one persistent launch over all of them.
cudaError_t enqueue_sweeps(Ctx* c, cudaStream_t st, bool multi)
{
    cudaError_t e;
    if (multi) {
        for (const Group& grp : c->G)
            if (c->wolff && (e = enqueue_wolff(c, grp, st)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(c->d_queue, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
        MultiArgs m{};
        m.a = group_args(c, c->G[0]);  // group 0 starts at configuration 0: conf_base as is
        m.groups = c->d_gdesc;
        m.tasks = c->d_tasks;
        m.ntasks = c->ntasks;
        m.queue = c->d_queue;
        return launch_multi(m, c->vac, c->multi_grid, st, false);
    }
    if (c->G.size() == 1) {
        const Group& grp = c->G[0];
        return enqueue_group(c, grp, grp.var, grp.nthreads, grp.smem, group_args(c, grp),
                             grp.nlat(), st, true);
    }
    if ((e = cudaEventRecord(c->fork_ev, st)) != cudaSuccess) return e;
    for (size_t k = 0; k < c->G.size(); ++k) {
        const Group& grp = c->G[k];
        if ((e = cudaStreamWaitEvent(c->side[k], c->fork_ev, 0)) != cudaSuccess) return e;
        e = enqueue_group(c, grp, grp.var, grp.nthreads, grp.smem, group_args(c, grp),
                          grp.nlat(), c->side[k], true);
        if (e != cudaSuccess) return e;
        if ((e = cudaEventRecord(c->join_ev[k], c->side[k])) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(st, c->join_ev[k], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// one PT cycle: every group's sweeps + observables, then swap / accumulate; with profiling,
// events e0 / e1 bracket the sweep launches
cudaError_t enqueue_cycle(Ctx* c, int measure, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1)
{
    cudaError_t e;
    // Several groups: the pair is recorded with or without profiling, so that one event node
    // heads the cycle's graph and one closes its branches before the swap (measured on the mixed
    // L = 16/24/32/48 batch: 403 attempts/ns with the two nodes, 382-396 with four root kernels
    // and a four-way join into the swap kernel)
    const bool rec = c->profile || c->G.size() > 1;
    if (rec && (e = cudaEventRecordWithFlags(e0, st, cudaEventRecordExternal)) != cudaSuccess)
        return e;
    if ((e = enqueue_sweeps(c, st, c->multi && multi_possible(c))) != cudaSuccess) return e;
    if (rec && (e = cudaEventRecordWithFlags(e1, st, cudaEventRecordExternal)) != cudaSuccess)
        return e;
    // one group without profiling events: the swap follows that group's last kernel directly
    const bool pdl = c->G.size() == 1 && !c->profile;
    if ((e = launch_swap(swap_args(c, measure), st, pdl)) != cudaSuccess) return e;
    if (measure && c->d_loc_s) return enqueue_locnem(c, st);
    return cudaSuccess;
}

int build_graph(Ctx* c, int measure)
{
    cudaGraph_t graph = nullptr;
    CK(c, cudaStreamBeginCapture(c->own, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_cycle(c, measure, c->own, c->ev0, c->ev1);
    cudaError_t e2 = cudaStreamEndCapture(c->own, &graph);
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(c, e, "capturing the PT-cycle graph");
    }
    if (e2 != cudaSuccess) return cuda_fail(c, e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->graph[measure], graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return cuda_fail(c, e, "cudaGraphInstantiate");
    }
    c->graph_src[measure] = graph;
    if (c->profile) {  // the two event-record nodes, retargeted to a pool pair per launch
        size_t n = 0;
        CK(c, cudaGraphGetNodes(graph, nullptr, &n));
        std::vector<cudaGraphNode_t> nodes(n);
        CK(c, cudaGraphGetNodes(graph, nodes.data(), &n));
        for (cudaGraphNode_t nd : nodes) {
            cudaGraphNodeType t;
            CK(c, cudaGraphNodeGetType(nd, &t));
            if (t != cudaGraphNodeTypeEventRecord) continue;
            cudaEvent_t ev = nullptr;
            CK(c, cudaGraphEventRecordNodeGetEvent(nd, &ev));
            if (ev == c->ev0) c->graph_ev[measure][0] = nd;
            if (ev == c->ev1) c->graph_ev[measure][1] = nd;
        }
        if (!c->graph_ev[measure][0] || !c->graph_ev[measure][1])
            return fail(c, J1J2C_ECUDA, "profiling events missing from the PT-cycle graph");
    }
    return J1J2C_OK;
}

bool valid_conf(Ctx* c, int conf) { return conf >= 0 && conf < c->nconf; }

// Autotuner: times every CTA size and form (one CTA per lattice, or streaming) of the
// shape-specialised kernel on a scratch copy of the group's lattices (the live state is not
// touched) and keeps the fastest.  Choices are cached per (device, precision, L, H, lattice
// count, vacancies) for the life of the process.
std::mutex g_tune_mu;
std::map<std::tuple<int, bool, int, int, int, bool>, int> g_tune_cache;

// Device time of 2 PT-cycle sweep launches of a group with kernel variant v (the fastest of three
// timings), on a scratch copy of its lattices (the live state is not touched; one warm-up launch
// first).  The launches are replays of a captured graph, as in a run, unless the context runs
// without graphs: variants with many small launches per cycle are timed as they run.
int time_variant(Ctx* c, Group& grp, const SweepVariant& v, int nthreads, size_t smem, float& ms)
{
    const int nlat = grp.nlat();
    uint8_t* tmp = nullptr;
    LatObs* tobs = nullptr;
    const size_t bytes = (size_t)nlat * grp.lat_stride;
    CK(c, dev_malloc(&tmp, bytes));
    if (dev_malloc(&tobs, sizeof(LatObs) * nlat) != cudaSuccess) {
        cudaFree(tmp);
        return fail(c, J1J2C_ENOMEM, "autotuner scratch");
    }
    cudaError_t e =
        cudaMemcpyAsync(tmp, c->d_spins + grp.spin_off, bytes, cudaMemcpyDeviceToDevice, c->own);
    SweepArgs a = group_args(c, grp);
    a.spins = tmp;
    a.obs = tobs;
    a.use_override = 1;
    a.beta_override = 1.0 / 9.5;
    a.sweep_override = 0x5EED0000u;
    a.flips = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess && !(c->P.flags & J1J2C_FLAG_NO_GRAPH)) {
        cudaGraph_t graph = nullptr;
        e = cudaStreamBeginCapture(c->own, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t e1 = enqueue_group(c, grp, v, nthreads, smem, a, nlat, c->own, false);
            e = cudaStreamEndCapture(c->own, &graph);
            if (e1 != cudaSuccess) e = e1;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
    }
    auto once = [&]() {
        return exec ? cudaGraphLaunch(exec, c->own)
                    : enqueue_group(c, grp, v, nthreads, smem, a, nlat, c->own, false);
    };
    // one untimed cycle, then one timed to size the timings: each covers at least about 1 ms of
    // cycles (a single small-batch cycle of tens of microseconds ranks candidates by launch
    // jitter)
    if (e == cudaSuccess) e = once();
    int reps = 2;
    {
        float t0 = 0.0f;
        if (e == cudaSuccess) e = cudaEventRecord(c->ev0, c->own);
        if (e == cudaSuccess) e = once();
        if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->own);
        if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t0, c->ev0, c->ev1);
        if (e == cudaSuccess && t0 > 0.0f && t0 < 0.5f) reps = std::min(64, (int)(1.0f / t0) + 1);
    }
    // the fastest of three timings (close candidates, noisy neighbours)
    ms = 0.0f;
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
        e = cudaEventRecord(c->ev0, c->own);
        for (int r = 0; r < reps && e == cudaSuccess; ++r) e = once();
        if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->own);
        if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
        float t = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, c->ev0, c->ev1);
        t /= (float)reps;  // per cycle: candidates are timed over different cycle counts
        if (e == cudaSuccess && (k == 0 || t < ms)) ms = t;
    }
    cudaStreamSynchronize(c->own);
    if (exec) cudaGraphExecDestroy(exec);
    cudaFree(tmp);
    cudaFree(tobs);
    if (e != cudaSuccess) return cuda_fail(c, e, "autotuning the sweep path");
    return J1J2C_OK;
}

// Cluster path or one launch per colour phase for a lattice that does not fit one CTA: the
// cluster kernel and the HBM kernel (shape-specialised form with 1, 2 or 4 replicas per thread
// where it exists, else the generic one) are timed and the fastest kept, cached per (device,
// precision, L, H, lattice count, bond dilution, HBM kernel).  Choice: 0 cluster, -1 generic HBM
// kernel, r > 0 shape-specialised HBM kernel with r replicas per thread.
std::map<std::tuple<int, bool, int, int, int, bool, int>, int> g_cluster_cache;

bool tune_log();  // J1J2C_TUNE_LOG=1: the tuners print their candidates' timings

int tune_cluster(Ctx* c, Group& grp)
{
    const int hbm_nt = hbm_fixed_threads(c, grp, grp.var.fp64);
    const auto key =
        std::make_tuple(c->P.device, grp.var.fp64, grp.g.L, grp.g.H, grp.nlat(), c->masks,
                        hbm_nt);
    int choice = 0;
    bool known = false;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_cluster_cache.find(key);
        if (it != g_cluster_cache.end()) {
            choice = it->second;
            known = true;
        }
    }
    if (!known) {
        float best_ms = 0.0f;
        int rc = time_variant(c, grp, grp.var, grp.nthreads, grp.smem, best_ms);
        if (rc != J1J2C_OK) return rc;
        SweepVariant vg = grp.var;
        vg.cluster = 0;
        vg.global = true;
        vg.stage_p = false;
        // CTA sizes of the shape's HBM kernels (the default first), else the generic kernel
        int sizes[4] = {0};
        const int nsz =
            hbm_nt > 0 ? fixed_hbm_sizes(grp.var.fp64, grp.g.L, grp.g.H, sizes, 4) : 1;
        // (eight replicas per thread, 128 registers and two CTAs per SM, measured slower at
        // L = 96: 5.41 vs 4.90 ms per Metropolis cycle of 8 x 48 lattices)
        for (int si = 0; si < nsz; ++si)
            for (int r = 1; r <= (sizes[si] > 0 ? 4 : 1); r *= 2) {
                if (grp.nrep % r) continue;
                vg.fixed_nt = sizes[si];
                vg.rpt = r;
                float ms = 0.0f;
                rc = time_variant(c, grp, vg, sizes[si] > 0 ? sizes[si] : 256, 0, ms);
                if (rc != J1J2C_OK) return rc;
                if (tune_log())
                    std::fprintf(stderr,
                                 "[j1j2c tune] lattices in HBM L=%d H=%d lattices=%d: %d threads, "
                                 "%d per thread %.3f ms (best before it %.3f ms)\n",
                                 grp.g.L, grp.g.H, grp.nlat(), sizes[si], r, ms, best_ms);
                if (ms < best_ms) {
                    best_ms = ms;
                    choice = sizes[si] > 0 ? (sizes[si] << 4 | r) : -1;  // CTA size and RPT
                }
            }
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_cluster_cache[key] = choice;
    }
    if (choice != 0) {
        const int nt = choice > 0 ? choice >> 4 : 0;
        grp.var.cluster = 0;
        grp.var.global = true;
        grp.var.stage_p = false;
        grp.var.fixed_nt = nt;
        grp.var.rpt = choice > 0 ? choice & 15 : 1;
        grp.smem = 0;
        grp.nthreads = nt > 0 ? nt : 256;
        free_graphs(c);
    }
    return J1J2C_OK;
}

// Generic global-memory kernels, one site per thread, nt threads per CTA
SweepVariant global_site_variant(const Ctx* c, bool fp64, int nt)
{
    SweepVariant v{};
    v.fp64 = fp64;
    v.masks = c->masks;
    v.vac = c->vac;
    v.mode = kModeSweep;
    v.global = true;
    v.rpt = 1;
    v.threads = nt;
    return v;
}

// The small-batch search applies to the default kernel choice only (the test flags pin a path)
bool small_batch_ok(Ctx* c, const Group& grp)
{
    return grp.block_threads == 0 && grp.var.mode == kModeSweep &&
           !(c->P.flags & (J1J2C_FLAG_GENERIC | J1J2C_FLAG_NO_FIXED | J1J2C_FLAG_GLOBAL |
                           J1J2C_FLAG_CLUSTER));
}

// Small batches (fewer lattices than half the SMs): one CTA per lattice leaves most SMs idle, so
// the chosen one-CTA kernel is timed against one site per thread in one CTA, every cluster size
// that divides H/2 (four sites or one site per thread), and one launch per colour phase with one
// site per thread in CTAs of 32-256 threads; the fastest is kept, cached per (device,
// precision, L, H, lattice count, bond dilution, vacancies).
enum SmallKind {
    kKeep = 0,
    kSiteCta = 1,
    kClusterQuad = 2,
    kClusterSite = 3,
    kGlobalSite = 4,
    kGlobalCoop = 5,  // kGlobalSite's phases in one cooperative launch
    kRepCluster = 6   // the lattice replicated in every CTA of a cluster of cs
};
struct SmallChoice {
    int kind, cs, nt;
};
std::map<std::tuple<int, bool, int, int, int, bool, bool>, SmallChoice> g_small_cache;

// The replicated-lattice cluster form with cs CTAs per lattice: one thread per site of a CTA's
// share of a colour (up to 1024 threads, which then loop)
SweepVariant rep_variant(Ctx* c, bool fp64, int cs, int L, int H)
{
    SweepVariant v{};
    v.fp64 = fp64;
    v.masks = c->masks;
    v.vac = c->vac;
    v.mode = kModeSweep;
    v.rep_cs = cs;
    const int per = (L / 2) * (L / 2) * (H / 2) / cs;
    v.threads = std::min(1024, ((per + 31) / 32) * 32);
    return v;
}

// Can the replicated-lattice form with cs CTAs per lattice run this group (shape divides, the
// cluster fits an SM set)?
bool rep_fits(Ctx* c, const Group& grp, int cs)
{
    if (grp.g.Nc % (4 * cs) != 0) return false;
    const SweepVariant v = rep_variant(c, grp.var.fp64, cs, grp.g.L, grp.g.H);
    const SweepArgs probe = group_args(c, grp);
    if (launch_sweep_rep(probe, v, grp.nlat(), nullptr, true) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return true;
}

// One site per thread in one CTA per lattice (the generic kernel)
int site_cta_variant(Ctx* c, Group& grp, SweepVariant& v, size_t& smem, int& nt)
{
    const uint32_t keep = c->P.flags;
    c->P.flags |= J1J2C_FLAG_GENERIC | J1J2C_FLAG_NO_FIXED;
    const int rc = choose_variant(c, grp, grp.var.fp64, v, smem, nt);
    c->P.flags = keep;
    nt = ((grp.g.Nc + 31) / 32) * 32;
    if (nt > 1024) nt = 1024;
    return rc;
}

SweepVariant cluster_variant(const SweepVariant& base, int cs, bool quad, int nt)
{
    SweepVariant v = base;
    v.cluster = cs;
    v.quad = quad;
    v.threads = nt;
    v.fixed_nt = 0;
    v.global = false;
    v.stage_p = false;
    return v;
}

int tune_small_batch(Ctx* c, Group& grp)
{
    int nsm = 0;
    CK(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->P.device));
    if (2 * grp.nlat() > nsm) return J1J2C_OK;
    const auto key =
        std::make_tuple(c->P.device, grp.var.fp64, grp.g.L, grp.g.H, grp.nlat(), c->masks,
                        c->vac);
    SmallChoice best{kKeep, 0, 0};
    bool known = false;
    if (c->P.flags & J1J2C_FLAG_COOP) {  // pinned: the cooperative form, 64 threads per CTA
        SweepVariant vc = global_site_variant(c, grp.var.fp64, 64);
        vc.coop = true;
        SweepArgs probe = group_args(c, grp);
        if (launch_sweep_coop(probe, vc, grp.nlat(), nullptr, nullptr, true) != cudaSuccess)
            return fail(c, J1J2C_EINVAL, "the cooperative form does not fit this batch");
        best = SmallChoice{kGlobalCoop, 0, 64};
        known = true;
    } else if (c->P.flags & J1J2C_FLAG_REPLICA) {
        // pinned: the largest cluster that fits, or J1J2C_REPLICA_CS from the environment (tests)
        const char* env = std::getenv("J1J2C_REPLICA_CS");
        const int want = env ? std::atoi(env) : 0;
        for (const int cs : {16, 8, 4, 2})
            if ((want == 0 || cs == want) && rep_fits(c, grp, cs)) {
                best = SmallChoice{kRepCluster, cs, 0};
                known = true;
                break;
            }
        if (!known) return fail(c, J1J2C_EINVAL, "the replicated-lattice form does not fit this batch");
    } else {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_small_cache.find(key);
        if (it != g_small_cache.end()) {
            best = it->second;
            known = true;
        }
    }
    if (!known) {
        float best_ms = 0.0f;
        int rc = time_variant(c, grp, grp.var, grp.nthreads, grp.smem, best_ms);
        if (rc != J1J2C_OK) return rc;
        if (tune_log())
            std::fprintf(stderr, "[j1j2c tune] small batch default nt=%d: %.4f ms\n",
                         grp.nthreads, best_ms);
        auto consider = [&](const SweepVariant& v, int nt, size_t smem, SmallChoice ch) {
            float ms = 0.0f;
            const int r = time_variant(c, grp, v, nt, smem, ms);
            if (tune_log())
                std::fprintf(stderr, "[j1j2c tune] small batch kind=%d cs=%d nt=%d: %.4f ms\n",
                             ch.kind, ch.cs, ch.nt, ms);
            if (r == J1J2C_OK && ms < best_ms) {
                best_ms = ms;
                best = ch;
            }
            return r;
        };
        // one site per thread (the latency of a colour phase is one site's arithmetic, not a
        // quad's: what counts for a handful of lattices)
        SweepVariant vs;
        size_t sm_s = 0;
        int nt_s = 0;
        if ((rc = site_cta_variant(c, grp, vs, sm_s, nt_s)) != J1J2C_OK) return rc;
        if (!vs.global && !vs.quad &&
            (rc = consider(vs, nt_s, sm_s, SmallChoice{kSiteCta, 0, nt_s})) != J1J2C_OK)
            return rc;
        int cs[16];
        const int n = cluster_sizes(grp.g, grp.var.fp64, c->masks, smem_budget(c), cs, 16);
        for (int k = 0; k < n; ++k) {
            const size_t sm = (size_t)grp.g.N / (size_t)cs[k];
            rc = consider(cluster_variant(grp.var, cs[k], true, 0), 512, sm,
                          SmallChoice{kClusterQuad, cs[k], 512});
            if (rc != J1J2C_OK) return rc;
            const int nt = cluster_site_threads(grp, cs[k]);
            rc = consider(cluster_variant(grp.var, cs[k], false, nt), nt, sm,
                          SmallChoice{kClusterSite, cs[k], nt});
            if (rc != J1J2C_OK) return rc;
        }
        // one launch per colour phase, one site per thread, small CTAs: the colour phase of a
        // handful of lattices spread over many SMs (the FP64 form is bound by each SM's FP64
        // rate, so the sites per SM, not per lattice, set its time)
        for (int nt = 32; nt <= 256; nt *= 2) {
            rc = consider(global_site_variant(c, grp.var.fp64, nt), nt, 0,
                          SmallChoice{kGlobalSite, 0, nt});
            if (rc != J1J2C_OK) return rc;
        }
        // (Not candidates: two forms with every sweep and the observables of a cycle in one
        // launch.  The cooperative form, grid barriers through L2 instead of kernel boundaries
        // (J1J2C_FLAG_COOP pins it), is slower on both the L = 16 single lattice and 16 lattices
        // of 24^3.  The replicated-lattice cluster form (J1J2C_FLAG_REPLICA; compile-time shape at
        // L = 16, 24) is at best 8 % faster in isolation on the single lattice, slower at 24^3,
        // and slower in the whole LOCAL cycle.  A colour phase of an FP64 small batch is bound by
        // one site's dependent chain (GB300: 64 clocks per dependent FP64 add or FMA), not by
        // its launch or barrier (a cluster barrier is ~0.2 us).)
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_small_cache[key] = best;
    }
    switch (best.kind) {
        case kClusterQuad:
        case kClusterSite:
            grp.var = cluster_variant(grp.var, best.cs, best.kind == kClusterQuad, best.nt);
            grp.smem = (size_t)grp.g.N / (size_t)best.cs;
            grp.nthreads = best.nt;
            break;
        case kGlobalSite:
        case kGlobalCoop:
            if (best.kind == kGlobalCoop && !c->d_gbar)
                CK(c, dalloc(&c->d_gbar, 2 * c->G.size()));
            grp.var = global_site_variant(c, grp.var.fp64, best.nt);
            grp.var.coop = best.kind == kGlobalCoop;
            grp.smem = 0;
            grp.nthreads = best.nt;
            break;
        case kSiteCta: {
            const int rc = site_cta_variant(c, grp, grp.var, grp.smem, grp.nthreads);
            if (rc != J1J2C_OK) return rc;
            break;
        }
        case kRepCluster:
            grp.var = rep_variant(c, grp.var.fp64, best.cs, grp.g.L, grp.g.H);
            grp.smem = rep_smem_bytes(grp.g, grp.var.fp64);
            grp.nthreads = grp.var.threads;
            break;
        default:
            return J1J2C_OK;
    }
    free_graphs(c);
    return J1J2C_OK;
}

// Wolff growth: 1, 2 or 4 CTAs per lattice (a thread-block cluster) for every lattice, or 2 CTAs
// for the 1/8, 1/4 or 1/2 coldest slots and one for the rest (two concurrent launches), timed on
// a scratch copy of the group's lattices at the first run of a context with Wolff updates, the
// fastest kept, cached per (device, precision, L, H, lattice count, bond dilution).  The coldest
// lattices' clusters span a third of the lattice or more and are bound by one SM's issue rate;
// the hot ones are small, and more CTAs per lattice mean more waves.
// J1J2C_TUNE_LOG=1 in the environment: the autotuners print every candidate's time to stderr
bool tune_log()
{
    const char* v = std::getenv("J1J2C_TUNE_LOG");
    return v && v[0] == '1';
}

struct WolffChoice {
    int cs, k;
};
std::map<std::tuple<int, bool, int, int, int, bool>, WolffChoice> g_wolff_cache;

constexpr int kWolffWarm = 40;  // cycles run on the Wolff tuner's scratch lattices before timing

int tune_wolff(Ctx* c, Group& grp)
{
    const uint32_t fl = c->P.flags;
    if (!c->wolff || (fl & (J1J2C_FLAG_GENERIC | J1J2C_FLAG_NO_FIXED | J1J2C_FLAG_WOLFF_CS2 |
                            J1J2C_FLAG_WOLFF_CS4 | J1J2C_FLAG_WOLFF_ASYNC)))
        return J1J2C_OK;  // no growth form, or the form is pinned
    const auto key =
        std::make_tuple(c->P.device, grp.var.fp64, grp.g.L, grp.g.H, grp.nlat(), c->masks);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_wolff_cache.find(key);
        if (it != g_wolff_cache.end()) {
            grp.wolff_cs = it->second.cs;
            grp.wolff_k = it->second.k;
            return J1J2C_OK;
        }
    }
    CK(c, alloc_labels(c));
    const int nlat = grp.nlat();
    uint8_t *tmp = nullptr, *snap = nullptr;
    LatObs* tobs = nullptr;
    uint32_t* wctl = nullptr;
    const size_t bytes = (size_t)nlat * grp.lat_stride;
    auto release = [&]() {
        cudaStreamSynchronize(c->own);
        for (void* p : {(void*)tmp, (void*)snap, (void*)tobs, (void*)wctl})
            if (p) cudaFree(p);
    };
    cudaError_t e = dev_malloc(&tmp, bytes);
    if (e == cudaSuccess) e = dev_malloc(&snap, bytes);
    if (e == cudaSuccess) e = dev_malloc(&tobs, sizeof(LatObs) * nlat);
    if (e == cudaSuccess) e = dev_malloc(&wctl, sizeof(uint32_t) * 4 * kWolffWarm);
    if (e != cudaSuccess) {  // no room for the scratch lattices: one CTA each, nothing cached
        release();
        cudaGetLastError();
        return J1J2C_OK;
    }
    e = cudaMemcpyAsync(tmp, c->d_spins + grp.spin_off, bytes, cudaMemcpyDeviceToDevice, c->own);
    SweepArgs a = group_args(c, grp);
    a.spins = tmp;
    // The scratch lattices first run kWolffWarm cycles (one-CTA Wolff update, sweeps and
    // observables) at their slots' temperatures: the clusters of a fresh start are far smaller
    // than those of an equilibrated cold lattice, which decide the choice.  Each warm-up cycle
    // reads its own cycle counter, so the random streams move on as in a run.  Every candidate
    // then starts from this state (restored from a second copy), so all of them are timed on
    // the same clusters: the forms flip the same clusters, so they also pass through the same
    // states while timed.
    if (e == cudaSuccess) {
        std::vector<uint32_t> h(4 * kWolffWarm, 0u);
        for (int r = 0; r < kWolffWarm; ++r) h[4 * r] = 0x7B000000u + (uint32_t)r;
        e = cudaMemcpy(wctl, h.data(), h.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    }
    for (int r = 0; r < kWolffWarm && e == cudaSuccess; ++r) {
        SweepArgs b = a;
        b.ctl = wctl + 4 * r;
        b.obs = tobs;
        b.flips = nullptr;
        e = enqueue_wolff_grow(c, grp, b, 1, 0, c->own);
        if (e == cudaSuccess)
            e = enqueue_group(c, grp, grp.var, grp.nthreads, grp.smem, b, nlat, c->own, false);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(snap, tmp, bytes, cudaMemcpyDeviceToDevice, c->own);
    // candidates (CTAs per lattice, coldest slots that take them; k = nrep: every slot)
    struct Cand {
        int cs, k;
    };
    // (the level-free growth is not a candidate: as fast as the level-synchronous form on
    // equilibrated L = 96 lattices, whose growth is bound by each cluster site's Philox work,
    // and ~4x slower on small clusters; J1J2C_FLAG_WOLFF_ASYNC pins it)
    std::vector<Cand> cands{{1, grp.nrep}, {2, grp.nrep}, {4, grp.nrep}};
    if (grp.nrep >= 8)
        for (const int k : {grp.nrep / 8, grp.nrep / 4, grp.nrep / 2}) cands.push_back({2, k});
    int best = 1, best_k = 0;
    float best_ms = 0.0f;
    for (const Cand cd : cands) {
        const int cs = cd.cs;
        if (e != cudaSuccess) break;
        if (cs > 1 && wolff_grow_clusters(grp.var.fp64, c->masks, cs) <= 0) continue;
        auto once = [&]() { return enqueue_wolff_grow(c, grp, a, cs, cd.k, c->own); };
        e = cudaMemcpyAsync(tmp, snap, bytes, cudaMemcpyDeviceToDevice, c->own);
        if (e == cudaSuccess) e = once();  // warm-up
        float ms = 0.0f;
        for (int k = 0; k < 3 && e == cudaSuccess; ++k) {  // the fastest of three
            e = cudaEventRecord(c->ev0, c->own);
            if (e == cudaSuccess) e = once();
            if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->own);
            if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
            float t = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, c->ev0, c->ev1);
            if (e == cudaSuccess && (k == 0 || t < ms)) ms = t;
        }
        if (tune_log())
            std::fprintf(stderr, "[j1j2c tune] wolff cs=%d k=%d: %.4f ms\n", cs, cd.k, ms);
        if (e == cudaSuccess && (cs == 1 || ms < best_ms)) {
            best_ms = ms;
            best = cs;
            best_k = cd.k < grp.nrep ? cd.k : 0;
        }
    }
    release();
    if (e != cudaSuccess) return cuda_fail(c, e, "autotuning the Wolff update");
    grp.wolff_cs = best;
    grp.wolff_k = best_k;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_wolff_cache[key] = WolffChoice{best, best_k};
    return J1J2C_OK;
}

// Split Wolff + sweep form (lattices in HBM with Wolff): the whole cycle's Wolff update, sweeps
// and observables timed on a scratch copy of the group's lattices (the live state is not
// touched), equilibrated by kSplitWarm cycles and restored before each candidate: unsplit, and
// split into two or more temperature ranges (the lists below), one CTA per cluster; the fastest
// is kept, cached per (device, precision, L, H, lattice count, dilution).  Two CTAs per cold
// cluster are not candidates: on a fresh HOT start (small clusters) they time fastest, on
// equilibrated lattices they are slower (L = 96, 8 x 48, two ranges: 11.0-12.4 vs 9.6 ms; the
// coldest of several ranges: 8.11 vs 7.88 ms).

// "k1,k2,..." of a 0-ended list of split points ("0": unsplit)
std::string pts_str(const int* pts)
{
    std::string out;
    for (int j = 0; j < kSplitRanges - 1 && (j == 0 || pts[j] > 0); ++j)
        out += (j ? "," : "") + std::to_string(pts[j]);
    return out;
}

// A split choice: the split points, cs CTAs per cluster of the coldest range, the coldest
// range's (unsplit: every slot's) bond activations decided beforehand
struct SplitChoice {
    int pts[kSplitRanges - 1];  // split points, a 0 ending the list (pts[0] = 0: unsplit)
    int cs;
    bool bits;
};
constexpr int kSplitWarm = 40;  // cycles run on the tuner's scratch lattices before timing
std::map<std::tuple<int, bool, int, int, int, bool>, SplitChoice> g_split_cache;

int tune_split(Ctx* c, Group& grp)
{
    const uint32_t fl = c->P.flags;
    if (!c->wolff || !grp.var.global || grp.var.fixed_nt <= 0 || grp.nrep < 8 ||
        (fl & (J1J2C_FLAG_GENERIC | J1J2C_FLAG_NO_FIXED | J1J2C_FLAG_WOLFF_CS2 |
               J1J2C_FLAG_WOLFF_CS4 | J1J2C_FLAG_WOLFF_SPLIT | J1J2C_FLAG_WOLFF_BITS |
               J1J2C_FLAG_NO_GRAPH)))
        return J1J2C_OK;
    const auto key =
        std::make_tuple(c->P.device, grp.var.fp64, grp.g.L, grp.g.H, grp.nlat(), c->masks);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_split_cache.find(key);
        if (it != g_split_cache.end()) {
            for (int j = 0; j < kSplitRanges - 1; ++j) grp.split[j] = it->second.pts[j];
            grp.split_cs = it->second.cs;
            grp.split_bits = it->second.bits;
            return J1J2C_OK;
        }
    }
    CK(c, alloc_labels(c));
    const int nlat = grp.nlat();
    uint8_t *tmp = nullptr, *snap = nullptr;
    LatObs* tobs = nullptr;
    uint32_t* wctl = nullptr;
    const size_t bytes = (size_t)nlat * grp.lat_stride;
    auto release = [&]() {
        cudaStreamSynchronize(c->own);
        for (void* p : {(void*)tmp, (void*)snap, (void*)tobs, (void*)wctl})
            if (p) cudaFree(p);
    };
    if (dev_malloc(&tmp, bytes) != cudaSuccess || dev_malloc(&snap, bytes) != cudaSuccess ||
        dev_malloc(&tobs, sizeof(LatObs) * nlat) != cudaSuccess ||
        dev_malloc(&wctl, sizeof(uint32_t) * 4 * kSplitWarm) != cudaSuccess) {
        release();  // no room for the scratch lattices: the cycle stays unsplit, nothing cached
        cudaGetLastError();
        return J1J2C_OK;
    }
    cudaError_t e =
        cudaMemcpyAsync(tmp, c->d_spins + grp.spin_off, bytes, cudaMemcpyDeviceToDevice, c->own);
    SweepArgs a = group_args(c, grp);
    a.spins = tmp;
    a.obs = tobs;
    a.flips = nullptr;
    // the cycle of one candidate, captured as a graph (as in a run)
    // one cycle of a candidate (the Wolff update, PTSWAPEVER sweeps, the observables) with
    // arguments b, enqueued on the context's stream
    auto enqueue = [&](const SplitChoice& cd, const SweepArgs& b) {
        if (cd.pts[0] > 0)
            return enqueue_split(c, grp, grp.var, b, cd.pts, cd.cs, c->own, cd.bits);
        grp.split_bits = cd.bits;  // read by enqueue_wolff_grow
        cudaError_t e1 = enqueue_wolff_grow(c, grp, b, wolff_cs_of(c, grp), wolff_k_of(c, grp),
                                            c->own);
        grp.split_bits = false;
        if (e1 == cudaSuccess)
            e1 = enqueue_group(c, grp, grp.var, grp.nthreads, grp.smem, b, nlat, c->own, false);
        return e1;
    };
    auto capture = [&](const SplitChoice& cd, cudaGraphExec_t& exec) {
        cudaGraph_t graph = nullptr;
        exec = nullptr;
        cudaError_t r = cudaStreamBeginCapture(c->own, cudaStreamCaptureModeThreadLocal);
        if (r == cudaSuccess) {
            const cudaError_t e1 = enqueue(cd, a);
            r = cudaStreamEndCapture(c->own, &graph);
            if (e1 != cudaSuccess) r = e1;
        }
        if (r == cudaSuccess) r = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        return r;
    };
    // (the cold slots' growth from bond activations decided beforehand, bits = true, measured
    // slower on equilibrated L = 96 lattices at every split and is left to its test flag)
    // split points between 1/4 and 3/4 of the slots: every multiple of 4 there when the ladder
    // is (the slot-range sweep kernel keeps four replicas per thread only when they divide the
    // range; L = 96, 48 slots: 8.88 ms at 28 vs 9.03 at 24 and 9.22 at 36), else eighths
    std::vector<SplitChoice> cands{{{}, 1, false}};
    auto push = [&](const SplitChoice& cd) {  // once each
        for (const SplitChoice& o : cands)
            if (std::equal(o.pts, o.pts + kSplitRanges - 1, cd.pts)) return;
        cands.push_back(cd);
    };
    auto two = [&](int k) {  // two ranges, split at k
        if (k > 0 && k < grp.nrep) push({{k}, 1, false});
    };
    if (grp.nrep % 4 == 0 && grp.nrep >= 16)
        for (int k = grp.nrep / 4; k <= 3 * grp.nrep / 4; k += 4) two(k - k % 4);
    else
        for (const int k8 : {2, 3, 4, 5, 6}) two(k8 * grp.nrep / 8);
    // more ranges: the coldest 4 or 8 slots alone, so that their long growths are followed by
    // the sweeps of few lattices, then ranges 8 slots wide up to a last boundary kl, and the
    // hottest slots from kl (L = 96, 8 x 48: 7.84 ms at 8,16,24,32,36 and 7.90-7.96 ms for five
    // other lists of this family, 8.63 ms at 32 alone; ranges 4 or 6 slots wide, and a coldest
    // range of 2 or 6 slots, were no faster)
    if (grp.nrep % 4 == 0 && grp.nrep >= 32)
        for (int kl = grp.nrep / 2 + 8; kl <= grp.nrep / 2 + 16; kl += 4)
            for (int c0 = 4; c0 <= 8; c0 += 4)
                for (int n = 1; c0 + (n - 1) * 8 < kl && n < kSplitRanges - 1; ++n) {
                    SplitChoice cd{{}, 1, false};
                    for (int i = 0; i < n; ++i) cd.pts[i] = c0 + i * 8;
                    cd.pts[n] = kl;
                    push(cd);
                }
    // The scratch lattices first run kSplitWarm cycles of the unsplit form at their slots'
    // temperatures (the clusters of a freshly started lattice are far smaller than those of an
    // equilibrated cold one, which decide the choice); each of these cycles reads its own cycle
    // counter, so the random stream moves on as in a run
    if (e == cudaSuccess) {
        std::vector<uint32_t> h(4 * kSplitWarm, 0u);
        for (int r = 0; r < kSplitWarm; ++r) h[4 * r] = 0x7A000000u + (uint32_t)r;
        e = cudaMemcpy(wctl, h.data(), h.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    }
    for (int r = 0; r < kSplitWarm && e == cudaSuccess; ++r) {
        SweepArgs b = a;
        b.ctl = wctl + 4 * r;
        e = enqueue(cands[0], b);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->own);
    // every candidate starts from the warmed state: the forms give the same lattices bit for
    // bit, so all of them are timed on the same clusters
    if (e == cudaSuccess) e = cudaMemcpyAsync(snap, tmp, bytes, cudaMemcpyDeviceToDevice, c->own);
    SplitChoice best = cands[0];
    float best_ms = 0.0f;
    for (size_t ci = 0; ci < cands.size(); ++ci) {
        const SplitChoice cd = cands[ci];
        if (e != cudaSuccess) break;
        cudaGraphExec_t exec = nullptr;
        e = capture(cd, exec);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(tmp, snap, bytes, cudaMemcpyDeviceToDevice, c->own);
        if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->own);  // warm-up
        float ms = 0.0f;
        for (int r = 0; r < 3 && e == cudaSuccess; ++r) {  // the fastest of three
            e = cudaEventRecord(c->ev0, c->own);
            if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->own);
            if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->own);
            if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
            float t = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, c->ev0, c->ev1);
            if (e == cudaSuccess && (r == 0 || t < ms)) ms = t;
        }
        if (exec) cudaGraphExecDestroy(exec);
        if (e == cudaSuccess && tune_log())
            std::fprintf(stderr,
                         "[j1j2c tune] split L=%d H=%d lattices=%d: at %s cs=%d bits=%d %.3f "
                         "ms\n",
                         grp.g.L, grp.g.H, nlat, pts_str(cd.pts).c_str(), cd.cs, (int)cd.bits,
                         ms);
        if (e == cudaSuccess && (ci == 0 || ms < best_ms)) {
            best_ms = ms;
            best = cd;
        }
    }
    cudaStreamSynchronize(c->own);
    release();
    if (e != cudaSuccess) return cuda_fail(c, e, "autotuning the split Wolff + sweep form");
    for (int j = 0; j < kSplitRanges - 1; ++j) grp.split[j] = best.pts[j];
    grp.split_cs = best.cs;
    grp.split_bits = best.bits;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_split_cache[key] = best;
    return J1J2C_OK;
}

// Device tables of the persistent multi-shape launch: one descriptor per group and the tile
// queue, groups with the largest tiles first (a longest-first order, so the last tiles to start
// are the shortest ones)
int setup_multi(Ctx* c)
{
    if (c->d_gdesc) return J1J2C_OK;
    const size_t ng = c->G.size();
    std::vector<GroupDesc> gd(ng);
    std::vector<int> order(ng);
    std::vector<long long> work(ng);
    for (size_t k = 0; k < ng; ++k) {
        const Group& grp = c->G[k];
        GroupDesc& d = gd[k];
        d.spins = c->d_spins + grp.spin_off;
        d.pf = c->d_pf + grp.p_off;
        d.lat_stride = grp.lat_stride;
        d.p_stride = grp.p_stride;
        d.beta = c->d_beta + grp.rep0;
        d.tor = c->d_tor + grp.rep0;
        d.obs = c->d_obs + grp.rep0;
        d.nrep = grp.nrep;
        d.conf0 = grp.conf0;
        d.kind = multi_tile_kind(grp.g.L, grp.g.H);
        order[k] = (int)k;
        work[k] = (long long)multi_tile_lattices(d.kind) * grp.g.N;
    }
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work[x] > work[y]; });
    std::vector<int2> tasks;
    for (const int k : order) {
        const int r = multi_tile_lattices(gd[k].kind);
        for (int l = 0; l < c->G[k].nlat(); l += r) tasks.push_back(make_int2(k, l));
    }
    int dev = 0, nsm = 0;
    CK(c, cudaGetDevice(&dev));
    CK(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    CK(c, dalloc(&c->d_gdesc, ng));
    CK(c, dalloc(&c->d_tasks, tasks.size()));
    CK(c, dalloc(&c->d_queue, 1));
    CK(c, cudaMemcpy(c->d_gdesc, gd.data(), ng * sizeof(GroupDesc), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_tasks, tasks.data(), tasks.size() * sizeof(int2),
                     cudaMemcpyHostToDevice));
    c->ntasks = (int)tasks.size();
    c->multi_grid = nsm < c->ntasks ? nsm : c->ntasks;
    MultiArgs none{};
    CK(c, launch_multi(none, c->vac, 0, nullptr, true));
    return J1J2C_OK;
}

// One persistent launch over every group, or one graph branch per group: at the first run the
// sweeps of one cycle in both forms are timed as graph replays on the live lattices (the fastest
// of three), whose spins, observables and cluster sizes are then put back; the faster form is
// kept for the life of the context.  Both give the same results bit for bit.
int tune_multi(Ctx* c)
{
    if (c->multi_tuned) return J1J2C_OK;
    c->multi_tuned = true;
    c->multi = false;
    if (!multi_possible(c)) return J1J2C_OK;
    {
        const int rc = setup_multi(c);
        if (rc != J1J2C_OK) return rc;
    }
    if (c->P.flags & J1J2C_FLAG_MULTI) {
        c->multi = true;
        free_graphs(c);
        return J1J2C_OK;
    }
    if (c->P.flags & J1J2C_FLAG_NO_GRAPH) return J1J2C_OK;
    if (c->wolff) CK(c, alloc_labels(c));
    const size_t ne = (size_t)c->nentries;
    uint8_t* keep_s = nullptr;
    LatObs* keep_o = nullptr;
    long long* keep_c = nullptr;
    cudaError_t e = dev_malloc(&keep_s, (size_t)c->spin_bytes);
    if (e == cudaSuccess) e = dev_malloc(&keep_o, ne * sizeof(LatObs));
    if (e == cudaSuccess) e = dev_malloc(&keep_c, ne * sizeof(long long));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(keep_s, c->d_spins, (size_t)c->spin_bytes, cudaMemcpyDeviceToDevice,
                            c->own);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(keep_o, c->d_obs, ne * sizeof(LatObs), cudaMemcpyDeviceToDevice,
                            c->own);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(keep_c, c->d_csize, ne * sizeof(long long),
                            cudaMemcpyDeviceToDevice, c->own);
    float ms[2] = {0.0f, 0.0f};
    for (int form = 0; form < 2 && e == cudaSuccess; ++form) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        e = cudaStreamBeginCapture(c->own, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t e1 = enqueue_sweeps(c, c->own, form == 1);
            e = cudaStreamEndCapture(c->own, &graph);
            if (e1 != cudaSuccess) e = e1;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->own);  // warm-up
        for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
            e = cudaEventRecord(c->ev0, c->own);
            if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->own);
            if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->own);
            if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
            float t = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, c->ev0, c->ev1);
            if (e == cudaSuccess && (r == 0 || t < ms[form])) ms[form] = t;
        }
        if (exec) cudaGraphExecDestroy(exec);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->d_spins, keep_s, (size_t)c->spin_bytes, cudaMemcpyDeviceToDevice,
                            c->own);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->d_obs, keep_o, ne * sizeof(LatObs), cudaMemcpyDeviceToDevice,
                            c->own);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->d_csize, keep_c, ne * sizeof(long long),
                            cudaMemcpyDeviceToDevice, c->own);
    cudaStreamSynchronize(c->own);
    cudaFree(keep_s);
    cudaFree(keep_o);
    cudaFree(keep_c);
    if (e != cudaSuccess) return cuda_fail(c, e, "autotuning the multi-shape launch");
    if (tune_log())
        std::fprintf(stderr, "j1j2c tune multi-shape sweeps: branches %.3f ms, one launch %.3f ms\n",
                     ms[0], ms[1]);
    c->multi = ms[1] < ms[0];
    free_graphs(c);
    return J1J2C_OK;
}

int autotune(Ctx* c, Group& grp)
{
    if (grp.tuned) return J1J2C_OK;
    grp.tuned = true;
    {
        const int rc = tune_wolff(c, grp);
        if (rc != J1J2C_OK) return rc;
    }
    if (c->P.flags & J1J2C_FLAG_CLUSTER) return J1J2C_OK;
    if (grp.var.cluster > 0 && grp.block_threads == 0) {
        const int rc = tune_cluster(c, grp);
        return rc != J1J2C_OK ? rc : tune_split(c, grp);
    }
    if (grp.var.global && grp.var.fixed_nt > 0) return tune_split(c, grp);  // HBM form pinned
    if (grp.block_threads > 0 || (c->P.flags & (J1J2C_FLAG_STREAM | J1J2C_FLAG_PAIRS)))
        return J1J2C_OK;
    if (grp.var.fixed_nt == 0) return small_batch_ok(c, grp) ? tune_small_batch(c, grp) : J1J2C_OK;
    FixedChoice fc[16];
    const int n = fixed_candidates(grp.var.fp64, grp.g.L, grp.g.H, c->masks, c->vac,
                                   int_couplings(c), grp.nrep, fc, 16);
    if (n <= 1) return small_batch_ok(c, grp) ? tune_small_batch(c, grp) : J1J2C_OK;
    const int nlat = grp.nlat();
    const auto key = std::make_tuple(c->P.device, grp.var.fp64, grp.g.L, grp.g.H, nlat, c->vac);
    int best = -1;  // index into fc
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) best = it->second;
    }
    const size_t budget = smem_budget(c);
    if (best < 0 || best >= n) {
        best = 0;
        uint8_t* tmp = nullptr;
        LatObs* tobs = nullptr;
        const size_t bytes = (size_t)nlat * grp.lat_stride;
        CK(c, dev_malloc(&tmp, bytes));
        if (dev_malloc(&tobs, sizeof(LatObs) * nlat) != cudaSuccess) {
            cudaFree(tmp);
            return fail(c, J1J2C_ENOMEM, "autotuner scratch");
        }
        cudaError_t e = cudaMemcpyAsync(tmp, c->d_spins + grp.spin_off, bytes,
                                        cudaMemcpyDeviceToDevice, c->own);
        SweepArgs a = group_args(c, grp);
        a.spins = tmp;
        a.obs = tobs;
        a.use_override = 1;
        a.beta_override = 1.0 / 9.5;
        a.sweep_override = 0x5EED0000u;
        float best_ms = 1e30f;
        for (int k = 0; k < n && e == cudaSuccess; ++k) {
            SweepVariant v = grp.var;
            v.fixed_nt = fc[k].nt;
            v.stage_p = fc[k].stage_p;
            v.stream = fc[k].stream;
            v.minb = fc[k].minb;
            v.rpc = fc[k].rpc;
            const size_t sm = sweep_smem_bytes(grp.g, v);
            if (sm > budget) continue;
            if ((e = launch_fixed(a, v.fp64, c->vac, fc[k], 0, sm, nullptr, true)) != cudaSuccess)
                break;
            if ((e = launch_fixed(a, v.fp64, c->vac, fc[k], nlat, sm, c->own, false)) !=
                cudaSuccess)
                break;
            cudaEventRecord(c->ev0, c->own);
            for (int r = 0; r < 3 && e == cudaSuccess; ++r)
                e = launch_fixed(a, v.fp64, c->vac, fc[k], nlat, sm, c->own, false);
            cudaEventRecord(c->ev1, c->own);
            if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            if (e == cudaSuccess && tune_log())
                std::fprintf(stderr,
                             "[j1j2c tune] sweep L=%d H=%d lattices=%d: nt=%d minb=%d stream=%d "
                             "rpc=%d %.4f ms\n",
                             grp.g.L, grp.g.H, nlat, fc[k].nt, fc[k].minb, (int)fc[k].stream,
                             fc[k].rpc, ms / 3.0f);
            if (e == cudaSuccess && ms < best_ms) {
                best_ms = ms;
                best = k;
            }
        }
        cudaStreamSynchronize(c->own);
        cudaFree(tmp);
        cudaFree(tobs);
        if (e != cudaSuccess) return cuda_fail(c, e, "autotuning the sweep kernel");
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best;
    }
    grp.var.fixed_nt = fc[best].nt;
    grp.var.stage_p = fc[best].stage_p;
    grp.var.stream = fc[best].stream;
    grp.var.minb = fc[best].minb;
    grp.var.rpc = fc[best].rpc;
    grp.smem = sweep_smem_bytes(grp.g, grp.var);
    grp.nthreads = fc[best].nt;
    {
        SweepArgs none{};
        none.g = grp.g;
        CK(c, launch_fixed(none, grp.var.fp64, c->vac, fc[best], 0, grp.smem, nullptr, true));
    }
    free_graphs(c);
    return small_batch_ok(c, grp) ? tune_small_batch(c, grp) : J1J2C_OK;
}

int check_params(const j1j2c_params* p, std::string& why)
{
    if (p->L < 2 || p->H < 2 || (p->L & 1) || (p->H & 1)) {
        why = "L and H must be even and >= 2 (8-colour update)";
        return J1J2C_EINVAL;
    }
    if ((long long)p->L * p->L * p->H > (1ll << 28)) {
        why = "lattice too large";
        return J1J2C_EINVAL;
    }
    if (p->nconf < 1 || p->nreplica < 1) {
        why = "nconf and nreplica must be >= 1";
        return J1J2C_EINVAL;
    }
    if (p->block_threads < 0 || p->block_threads > 1024 || (p->block_threads % 32)) {
        why = "block_threads must be 0 or a multiple of 32 up to 1024";
        return J1J2C_EINVAL;
    }
    return J1J2C_OK;
}

Geo make_geo(int L, int H)
{
    Geo g{};
    g.L = L;
    g.H = H;
    g.Lh = L / 2;
    g.Hh = H / 2;
    g.N = L * L * H;
    g.Nc = g.Lh * g.Lh * g.Hh;
    g.Qr = (g.Lh + 3) / 4;
    return g;
}

}  // namespace

extern "C" {

const char* j1j2c_version(void) { return "j1j2cuda 0.2 (sm_103a)"; }

const char* j1j2c_last_error(void* ctx)
{
    if (!ctx) return g_create_error.c_str();
    return static_cast<Ctx*>(ctx)->err.c_str();
}

int j1j2c_create_multi(void** out, const j1j2c_params* groups, int32_t ngroups)
{
    g_create_error.clear();
    if (!out || !groups || ngroups < 1 || ngroups > 64) {
        g_create_error = "null argument or bad group count";
        return J1J2C_EINVAL;
    }
    *out = nullptr;
    const j1j2c_params* p = &groups[0];
    auto bad = [](const std::string& m) {
        g_create_error = m;
        return J1J2C_EINVAL;
    };
    for (int k = 0; k < ngroups; ++k) {
        std::string why;
        if (check_params(&groups[k], why) != J1J2C_OK) return bad(why);
    }
    if (p->ptswapever < 1) return bad("ptswapever must be positive (J:909-912)");
    if (p->precision != J1J2C_FP64_PLAIN && p->precision != J1J2C_FP32_BATCHED)
        return bad("precision must be J1J2C_FP64_PLAIN or J1J2C_FP32_BATCHED");
    if (!std::isfinite(p->J1h) || !std::isfinite(p->J1v) || !std::isfinite(p->J2) ||
        !std::isfinite(p->J3))
        return bad("couplings must be finite");

    Ctx* c = new Ctx();
    c->P = *p;
    long long spin_bytes = 0, p_elems = 0, mask_bytes = 0;
    for (int k = 0; k < ngroups; ++k) {
        Group grp;
        grp.g = make_geo(groups[k].L, groups[k].H);
        grp.nconf = groups[k].nconf;
        grp.nrep = groups[k].nreplica;
        grp.block_threads = groups[k].block_threads;
        grp.conf0 = c->nconf;
        grp.rep0 = c->nentries;
        grp.lat_stride = ((long long)grp.g.N + 15) & ~15ll;
        grp.p_stride = ((long long)grp.g.N + 3) & ~3ll;
        grp.spin_off = spin_bytes;
        grp.p_off = p_elems;
        grp.mask_off = mask_bytes;
        grp.lab_off = c->lab_ints;
        c->lab_ints += (long long)grp.nlat() * grp.lat_stride;
        spin_bytes += (long long)grp.nlat() * grp.lat_stride;
        p_elems += (long long)grp.nconf * grp.p_stride;
        mask_bytes += (long long)grp.nconf * grp.lat_stride;
        for (int j = 0; j < grp.nconf; ++j) {
            c->conf_group.push_back(k);
            c->conf_rbase.push_back(c->nentries + j * grp.nrep);
            c->conf_nrep.push_back(grp.nrep);
        }
        c->nconf += grp.nconf;
        c->nentries += grp.nlat();
        c->G.push_back(grp);
    }
    c->spin_bytes = spin_bytes;
    c->mask_bytes = mask_bytes;
    c->p_elems = p_elems;
    c->have_dis.assign(c->nconf, 0);
    c->have_ladder.assign(c->nconf, 0);
    c->have_spins.assign(c->nconf, 0);
    c->nocc.assign(c->nconf, 0);
    c->conf_masks.assign(c->nconf, 0);
    c->conf_vac.assign(c->nconf, 0);
    c->profile = (p->flags & J1J2C_FLAG_PROFILE) != 0;

    auto cfail = [&](cudaError_t e, const char* what) {
        g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
        release(c);
        delete c;
        return e == cudaErrorMemoryAllocation ? J1J2C_ENOMEM : J1J2C_ECUDA;
    };
    cudaError_t e = cudaSetDevice(p->device);
    if (e != cudaSuccess) return cfail(e, "cudaSetDevice");
    const size_t ne = (size_t)c->nentries, nc = (size_t)c->nconf;
    if ((e = dalloc(&c->d_spins, (size_t)spin_bytes)) != cudaSuccess) return cfail(e, "spins");
    if ((e = dalloc(&c->d_pf, (size_t)p_elems)) != cudaSuccess) return cfail(e, "field");
    if ((e = dalloc(&c->d_pd, (size_t)p_elems)) != cudaSuccess) return cfail(e, "field");
    if ((e = dalloc(&c->d_bm, (size_t)mask_bytes)) != cudaSuccess) return cfail(e, "masks");
    if ((e = dalloc(&c->d_occ, (size_t)mask_bytes)) != cudaSuccess) return cfail(e, "occ");
    if ((e = dalloc(&c->d_beta, ne)) != cudaSuccess) return cfail(e, "beta");
    if ((e = dalloc(&c->d_kb, ne)) != cudaSuccess) return cfail(e, "beta");
    if ((e = dalloc(&c->d_rat, ne)) != cudaSuccess) return cfail(e, "maps");
    if ((e = dalloc(&c->d_tor, ne)) != cudaSuccess) return cfail(e, "maps");
    if ((e = dalloc(&c->d_obs, ne)) != cudaSuccess) return cfail(e, "obs");
    if ((e = dalloc(&c->d_sums, ne * 22)) != cudaSuccess) return cfail(e, "sums");
    if ((e = dalloc(&c->d_nmeas, ne)) != cudaSuccess) return cfail(e, "sums");
    if ((e = dalloc(&c->d_att, ne)) != cudaSuccess) return cfail(e, "pt stats");
    if ((e = dalloc(&c->d_acc, ne)) != cudaSuccess) return cfail(e, "pt stats");
    if ((e = dalloc(&c->d_vis, ne)) != cudaSuccess) return cfail(e, "pt stats");
    if ((e = dalloc(&c->d_last, ne * 5)) != cudaSuccess) return cfail(e, "obs");
    if ((e = dalloc(&c->d_ctl, 4)) != cudaSuccess) return cfail(e, "ctl");
    if ((e = dalloc(&c->d_nocc, nc)) != cudaSuccess) return cfail(e, "nocc");
    if ((e = dalloc(&c->d_rbase, nc)) != cudaSuccess) return cfail(e, "rbase");
    if ((e = dalloc(&c->d_nreps, nc)) != cudaSuccess) return cfail(e, "nreps");
    if ((e = dalloc(&c->d_audit, 2)) != cudaSuccess) return cfail(e, "audit");
    if ((e = dalloc(&c->d_csize, ne)) != cudaSuccess) return cfail(e, "cluster sizes");
    if ((e = dalloc(&c->d_err, 1)) != cudaSuccess) return cfail(e, "error word");
    if ((e = cudaMemset(c->d_err, 0, sizeof(int))) != cudaSuccess) return cfail(e, "memset");
    if ((e = cudaMemset(c->d_csize, 0, ne * sizeof(long long))) != cudaSuccess)
        return cfail(e, "memset");
    c->wolff = (p->flags & J1J2C_FLAG_WOLFF) != 0;
    if ((e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking)) != cudaSuccess)
        return cfail(e, "stream");
    if (c->wolff && (e = alloc_labels(c)) != cudaSuccess) return cfail(e, "Wolff labels");
    c->st = c->own;
    if (ngroups > 1) {
        if ((e = cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming)) != cudaSuccess)
            return cfail(e, "event");
        for (int k = 0; k < ngroups; ++k) {
            cudaStream_t s;
            cudaEvent_t ev;
            if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess)
                return cfail(e, "stream");
            c->side.push_back(s);
            if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
                return cfail(e, "event");
            c->join_ev.push_back(ev);
        }
    }
    for (const Group& grp : c->G)
        if ((e = wolff_side(c, grp)) != cudaSuccess) return cfail(e, "Wolff stream");
    if ((e = cudaEventCreate(&c->ev0)) != cudaSuccess) return cfail(e, "event");
    if ((e = cudaEventCreate(&c->ev1)) != cudaSuccess) return cfail(e, "event");
    for (int k = 0; c->profile && k < kProfPool; ++k) {
        cudaEvent_t a = nullptr, b = nullptr;
        if ((e = cudaEventCreate(&a)) != cudaSuccess) return cfail(e, "event");
        c->pev0.push_back(a);
        if ((e = cudaEventCreate(&b)) != cudaSuccess) return cfail(e, "event");
        c->pev1.push_back(b);
    }
    if ((e = cudaMemset(c->d_spins, 1, (size_t)spin_bytes)) != cudaSuccess)
        return cfail(e, "memset");
    if ((e = cudaMemset(c->d_bm, 3, (size_t)mask_bytes)) != cudaSuccess) return cfail(e, "memset");
    if ((e = cudaMemset(c->d_obs, 0, ne * sizeof(LatObs))) != cudaSuccess)
        return cfail(e, "memset");
    if ((e = cudaMemcpy(c->d_ctl, c->host_ctl, 4 * sizeof(uint32_t), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
        return cfail(e, "ctl");
    if ((e = cudaMemcpy(c->d_rbase, c->conf_rbase.data(), nc * sizeof(int),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
        return cfail(e, "rbase");
    if ((e = cudaMemcpy(c->d_nreps, c->conf_nrep.data(), nc * sizeof(int),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
        return cfail(e, "nreps");
    for (auto& grp : c->G) {
        int rc = choose_variant(c, grp, p->precision == J1J2C_FP64_PLAIN, grp.var, grp.smem,
                                grp.nthreads);
        if (rc != J1J2C_OK) {
            g_create_error = c->err;
            release(c);
            delete c;
            return rc;
        }
    }
    *out = c;
    int rc = j1j2c_reset_measurements(c, -1);
    if (rc != J1J2C_OK) {
        g_create_error = c->err;
        release(c);
        delete c;
        *out = nullptr;
        return rc;
    }
    return J1J2C_OK;
}

int j1j2c_create(void** out, const j1j2c_params* p)
{
    if (!p) {
        g_create_error = "null argument";
        return J1J2C_EINVAL;
    }
    return j1j2c_create_multi(out, p, 1);
}

void j1j2c_destroy(void* ctx)
{
    if (!ctx) return;
    Ctx* c = static_cast<Ctx*>(ctx);
    cudaStreamSynchronize(c->st);
    release(c);
    delete c;
}

int j1j2c_set_stream(void* ctx, void* stream)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    c->st = stream ? static_cast<cudaStream_t>(stream) : c->own;
    return J1J2C_OK;
}

int j1j2c_conf_shape(void* ctx, int32_t conf, int32_t* L, int32_t* H, int32_t* nreplica)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    const Group& grp = c->G[c->conf_group[conf]];
    if (L) *L = grp.g.L;
    if (H) *H = grp.g.H;
    if (nreplica) *nreplica = grp.nrep;
    return J1J2C_OK;
}

int j1j2c_set_disorder(void* ctx, int32_t conf, const double* p, const int8_t* occu,
                       const int8_t* jh, const int8_t* jv)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    if (!p) return fail(c, J1J2C_EINVAL, "p is null");
    Group& grp = c->G[c->conf_group[conf]];
    const Geo& g = grp.g;
    std::vector<double> pd((size_t)grp.p_stride, 0.0);
    std::vector<float> pf((size_t)grp.p_stride, 0.0f);
    std::vector<uint8_t> occ((size_t)grp.lat_stride, 0), bm((size_t)grp.lat_stride, 3);
    int nocc = 0, anymask = 0;
    for (int s = 0; s < g.N; ++s) {
        if (!std::isfinite(p[s])) return fail(c, J1J2C_EINVAL, "p must be finite");
        const int ci = compact_of_site(g, s);
        pd[ci] = p[s];
        pf[ci] = (float)p[s];
        const int o = occu ? (occu[s] != 0) : 1;
        occ[ci] = (uint8_t)o;
        nocc += o;
        const int h = jh ? (jh[s] != 0) : 1, v = jv ? (jv[s] != 0) : 1;
        bm[ci] = (uint8_t)(h | (v << 1));
        anymask |= (h == 0 || v == 0);
    }
    const int lc = conf - grp.conf0;
    CK(c, cudaMemcpy(c->d_pd + grp.p_off + (size_t)lc * grp.p_stride, pd.data(), pd.size() * 8,
                     cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_pf + grp.p_off + (size_t)lc * grp.p_stride, pf.data(), pf.size() * 4,
                     cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_occ + grp.mask_off + (size_t)lc * grp.lat_stride, occ.data(),
                     occ.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_bm + grp.mask_off + (size_t)lc * grp.lat_stride, bm.data(), bm.size(),
                     cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_nocc + conf, &nocc, sizeof(int), cudaMemcpyHostToDevice));
    c->nocc[conf] = nocc;
    c->conf_masks[conf] = anymask;
    c->conf_vac[conf] = nocc < g.N;
    bool masks = false, vac = false;
    for (int k : c->conf_masks) masks = masks || k;
    for (int k : c->conf_vac) vac = vac || k;
    if (masks != c->masks || vac != c->vac) {
        c->masks = masks;
        c->vac = vac;
        free_graphs(c);
        for (auto& gr : c->G) {
            int rc = choose_variant(c, gr, c->P.precision == J1J2C_FP64_PLAIN, gr.var, gr.smem,
                                    gr.nthreads);
            if (rc != J1J2C_OK) return rc;
            gr.tuned = false;
        }
    }
    c->have_dis[conf] = 1;
    c->have_spins[conf] = 0;  // vacancies changed: spins must be initialised again
    c->occ_total = 0;
    for (int k = 0; k < c->nconf; ++k) c->occ_total += (long long)c->nocc[k] * c->conf_nrep[k];
    return J1J2C_OK;
}

// The FP32 form's acceptance scale of each beta, (float)(-2 beta log2(e)): the same IEEE double
// operations, in the same order, as the kernels that compute it themselves
std::vector<float> acceptance_scales(const double* beta, int n)
{
    std::vector<float> kb((size_t)n);
    for (int k = 0; k < n; ++k) kb[(size_t)k] = (float)(-2.0 * beta[k] * 1.4426950408889634);
    return kb;
}

int j1j2c_set_ladder(void* ctx, int32_t conf, const double* beta)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (conf >= c->nconf) return fail(c, J1J2C_EINVAL, "conf out of range");
    if (!beta) return fail(c, J1J2C_EINVAL, "beta is null");
    const int off = conf < 0 ? 0 : c->conf_rbase[conf];
    const int n = conf < 0 ? c->nentries : c->conf_nrep[conf];
    for (int k = 0; k < n; ++k)
        if (!std::isfinite(beta[k]) || beta[k] < 0.0)
            return fail(c, J1J2C_EINVAL, "beta must be finite and >= 0");
    CK(c, cudaMemcpyAsync(c->d_beta + off, beta, sizeof(double) * n, cudaMemcpyHostToDevice,
                          c->st));
    const std::vector<float> kb = acceptance_scales(beta, n);
    CK(c, cudaMemcpyAsync(c->d_kb + off, kb.data(), sizeof(float) * n, cudaMemcpyHostToDevice,
                          c->st));
    CK(c, cudaStreamSynchronize(c->st));
    if (conf < 0)
        for (int k = 0; k < c->nconf; ++k) c->have_ladder[k] = 1;
    else
        c->have_ladder[conf] = 1;
    return J1J2C_OK;
}

int j1j2c_init_spins(void* ctx, int32_t conf, int32_t start, int32_t axis, const int8_t* spins)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    if (!c->have_dis[conf]) return fail(c, J1J2C_ESTATE, "set_disorder must precede init_spins");
    if (!spins && (start < 0 || start > 2)) return fail(c, J1J2C_EINVAL, "START must be HOT/FER/STR");
    if (!spins && start == J1J2C_START_STR && axis != 0 && axis != 1)
        return fail(c, J1J2C_EINVAL, "STRAXIS must be X or Y");
    const Group& grp = c->G[c->conf_group[conf]];
    const Geo& g = grp.g;
    const int lc = conf - grp.conf0, nrep = grp.nrep;
    uint8_t* dst = c->d_spins + grp.spin_off + (size_t)lc * nrep * grp.lat_stride;
    const uint8_t* occd = c->d_occ + grp.mask_off + (size_t)lc * grp.lat_stride;
    if (spins) {
        std::vector<uint8_t> occ((size_t)g.N);
        CK(c, cudaMemcpy(occ.data(), occd, g.N, cudaMemcpyDeviceToHost));
        std::vector<uint8_t> buf((size_t)nrep * grp.lat_stride, 1);
        for (int r = 0; r < nrep; ++r)
            for (int s = 0; s < g.N; ++s) {
                const int8_t v = spins[(size_t)r * g.N + s];
                if (v != 1 && v != -1) return fail(c, J1J2C_EINVAL, "spins must be +1 or -1");
                const int ci = compact_of_site(g, s);
                buf[(size_t)r * grp.lat_stride + ci] = occ[ci] ? (uint8_t)(v + 1) : (uint8_t)1;
            }
        CK(c, cudaMemcpy(dst, buf.data(), buf.size(), cudaMemcpyHostToDevice));
    } else {
        InitArgs a{};
        a.g = g;
        a.spins = dst;
        a.lat_stride = grp.lat_stride;
        a.occ = occd;
        a.nrep = nrep;
        a.start = start;
        a.axis = axis;
        a.seed = c->P.seed;
        a.key1 = c->P.conf_base + (uint32_t)conf;
        CK(c, launch_init(a, c->st));
    }
    // Initialize_pt_state: identity maps, swap counters and flip counts zeroed (J:1222-1233)
    const int rb = c->conf_rbase[conf];
    if (c->d_flips)
        CK(c, cudaMemsetAsync(c->d_flips + grp.spin_off + (size_t)lc * nrep * grp.lat_stride, 0,
                              sizeof(int) * (size_t)nrep * grp.lat_stride, c->st));
    CK(c, cudaMemsetAsync(c->d_att + rb, 0, sizeof(long long) * nrep, c->st));
    CK(c, cudaMemsetAsync(c->d_acc + rb, 0, sizeof(long long) * nrep, c->st));
    std::vector<int> ident((size_t)nrep);
    for (int r = 0; r < nrep; ++r) ident[r] = r;
    CK(c, cudaMemcpyAsync(c->d_rat + rb, ident.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice,
                          c->st));
    CK(c, cudaMemcpyAsync(c->d_tor + rb, ident.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice,
                          c->st));
    CK(c, cudaStreamSynchronize(c->st));
    c->have_spins[conf] = 1;
    return J1J2C_OK;
}

int j1j2c_reset_measurements(void* ctx, int32_t conf)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (conf >= c->nconf) return fail(c, J1J2C_EINVAL, "conf out of range");
    const size_t off = conf < 0 ? 0 : (size_t)c->conf_rbase[conf];
    const size_t n = conf < 0 ? (size_t)c->nentries : (size_t)c->conf_nrep[conf];
    std::vector<double> sums(n * 22, 0.0);
    for (size_t k = 0; k < n; ++k) sums[k * 22 + 20] = std::numeric_limits<double>::infinity();
    CK(c, cudaMemcpy(c->d_sums + off * 22, sums.data(), sums.size() * 8, cudaMemcpyHostToDevice));
    CK(c, cudaMemset(c->d_nmeas + off, 0, n * sizeof(long long)));
    CK(c, cudaMemset(c->d_vis + off, 0, n));
    // histograms start again (range from the next first sample, J:1227-1230) and so do the
    // local nematic averages (Reset_local_nematic_average, J:1388)
    if (c->d_hist) {
        const size_t bins = (size_t)c->diag.hist_bins;
        CK(c, cudaMemset(c->d_hist + off * bins, 0, n * bins * sizeof(long long)));
        CK(c, cudaMemset(c->d_hist_bs + off, 0, n * sizeof(double)));
        CK(c, cudaMemset(c->d_hist_lo + off, 0, n * sizeof(double)));
    }
    if (c->d_loc_s) {
        size_t lo = 0, len = (size_t)c->mask_bytes;
        if (conf >= 0) {
            const Group& grp = c->G[c->conf_group[conf]];
            lo = (size_t)grp.mask_off + (size_t)(conf - grp.conf0) * grp.lat_stride;
            len = (size_t)grp.lat_stride;
        }
        CK(c, cudaMemset(c->d_loc_s + lo, 0, len * sizeof(int)));
        CK(c, cudaMemset(c->d_loc_n + lo, 0, len * sizeof(int)));
        CK(c, cudaMemset(c->d_loc_samples + (conf < 0 ? 0 : conf), 0,
                         (conf < 0 ? (size_t)c->nconf : 1) * sizeof(long long)));
    }
    return J1J2C_OK;
}

int j1j2c_set_diagnostics(void* ctx, const j1j2c_diagnostics* d)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!d) return fail(c, J1J2C_EINVAL, "null diagnostics");
    if (d->locnem_slot < -1 || d->hist_bins < 0 || d->hist_bins > (1 << 20) ||
        d->trace_cycles < 0 || (d->flip_counts != 0 && d->flip_counts != 1))
        return fail(c, J1J2C_EINVAL, "bad diagnostics settings");
    CK(c, cudaStreamSynchronize(c->st));
    free_graphs(c);
    auto drop = [](auto*& p) {
        if (p) cudaFree(p);
        p = nullptr;
    };
    drop(c->d_loc_s);
    drop(c->d_loc_n);
    drop(c->d_loc_samples);
    drop(c->d_hist);
    drop(c->d_hist_lo);
    drop(c->d_hist_bs);
    drop(c->d_trace);
    drop(c->d_trace_tor);
    drop(c->d_flips);
    const bool flips_changed = (d->flip_counts != 0) != (c->diag.flip_counts != 0);
    c->diag = *d;
    const size_t ne = (size_t)c->nentries;
    if (d->locnem_slot >= 0) {
        const size_t n = (size_t)c->mask_bytes;
        CK(c, dalloc(&c->d_loc_s, n));
        CK(c, dalloc(&c->d_loc_n, n));
        CK(c, dalloc(&c->d_loc_samples, (size_t)c->nconf));
        CK(c, cudaMemset(c->d_loc_s, 0, n * sizeof(int)));
        CK(c, cudaMemset(c->d_loc_n, 0, n * sizeof(int)));
        CK(c, cudaMemset(c->d_loc_samples, 0, (size_t)c->nconf * sizeof(long long)));
    }
    if (d->hist_bins > 0) {
        CK(c, dalloc(&c->d_hist, ne * (size_t)d->hist_bins));
        CK(c, dalloc(&c->d_hist_lo, ne));
        CK(c, dalloc(&c->d_hist_bs, ne));
        CK(c, cudaMemset(c->d_hist, 0, ne * (size_t)d->hist_bins * sizeof(long long)));
        CK(c, cudaMemset(c->d_hist_lo, 0, ne * sizeof(double)));
        CK(c, cudaMemset(c->d_hist_bs, 0, ne * sizeof(double)));
    }
    if (d->trace_cycles > 0) {
        CK(c, dalloc(&c->d_trace, (size_t)d->trace_cycles * ne * 5));
        CK(c, dalloc(&c->d_trace_tor, (size_t)d->trace_cycles * ne));
    }
    if (d->flip_counts) {
        CK(c, dalloc(&c->d_flips, (size_t)c->spin_bytes));
        CK(c, cudaMemset(c->d_flips, 0, (size_t)c->spin_bytes * sizeof(int)));
    }
    if (flips_changed)
        for (auto& gr : c->G) {
            int rc = choose_variant(c, gr, c->P.precision == J1J2C_FP64_PLAIN, gr.var, gr.smem,
                                    gr.nthreads);
            if (rc != J1J2C_OK) return rc;
            gr.tuned = false;
        }
    return J1J2C_OK;
}

int j1j2c_get_diagnostics(void* ctx, j1j2c_diagnostics* out)
{
    if (!ctx || !out) return J1J2C_EINVAL;
    *out = static_cast<Ctx*>(ctx)->diag;
    return J1J2C_OK;
}

int j1j2c_get_occupied(void* ctx, int32_t conf, int32_t* nocc)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf) || !nocc) return fail(c, J1J2C_EINVAL, "bad conf or null output");
    *nocc = c->nocc[conf];
    return J1J2C_OK;
}

int j1j2c_get_locnem(void* ctx, int32_t conf, double* locspin, double* locnem, int64_t* samples)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    if (!c->d_loc_s) return fail(c, J1J2C_ESTATE, "local nematic averages are not enabled");
    const Group& grp = c->G[c->conf_group[conf]];
    const Geo& g = grp.g;
    const size_t off = (size_t)grp.mask_off + (size_t)(conf - grp.conf0) * grp.lat_stride;
    std::vector<int> vs((size_t)g.N), vn((size_t)g.N);
    long long ns = 0;
    CK(c, cudaStreamSynchronize(c->st));
    CK(c, cudaMemcpy(vs.data(), c->d_loc_s + off, sizeof(int) * g.N, cudaMemcpyDeviceToHost));
    CK(c, cudaMemcpy(vn.data(), c->d_loc_n + off, sizeof(int) * g.N, cudaMemcpyDeviceToHost));
    CK(c, cudaMemcpy(&ns, c->d_loc_samples + conf, sizeof ns, cudaMemcpyDeviceToHost));
    for (int st = 0; st < g.N; ++st) {
        const int ci = compact_of_site(g, st);
        if (locspin) locspin[st] = (double)vs[ci];
        if (locnem) locnem[st] = (double)vn[ci];
    }
    if (samples) *samples = ns;
    return J1J2C_OK;
}

int j1j2c_get_histogram(void* ctx, int32_t conf, double* counts, double* emin, double* binsize)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    if (!c->d_hist) return fail(c, J1J2C_ESTATE, "the energy histogram is not enabled");
    const size_t off = (size_t)c->conf_rbase[conf], n = (size_t)c->conf_nrep[conf];
    const size_t bins = (size_t)c->diag.hist_bins;
    std::vector<long long> h(n * bins);
    CK(c, cudaStreamSynchronize(c->st));
    CK(c, cudaMemcpy(h.data(), c->d_hist + off * bins, h.size() * sizeof(long long),
                     cudaMemcpyDeviceToHost));
    if (counts)
        for (size_t k = 0; k < h.size(); ++k) counts[k] = (double)h[k];
    if (emin) CK(c, cudaMemcpy(emin, c->d_hist_lo + off, n * sizeof(double), cudaMemcpyDeviceToHost));
    if (binsize)
        CK(c, cudaMemcpy(binsize, c->d_hist_bs + off, n * sizeof(double), cudaMemcpyDeviceToHost));
    return J1J2C_OK;
}

int j1j2c_get_trace(void* ctx, int32_t conf, double* obs, int32_t* temp_of_rep, int64_t* ncycles)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    if (!c->d_trace) return fail(c, J1J2C_ESTATE, "the observable trace is not enabled");
    const size_t off = (size_t)c->conf_rbase[conf], n = (size_t)c->conf_nrep[conf];
    const size_t ne = (size_t)c->nentries;
    long long nm = 0;
    CK(c, cudaStreamSynchronize(c->st));
    CK(c, cudaMemcpy(&nm, c->d_nmeas + off, sizeof nm, cudaMemcpyDeviceToHost));
    const size_t rows = (size_t)(nm < c->diag.trace_cycles ? nm : c->diag.trace_cycles);
    if (rows > 0 && obs)
        CK(c, cudaMemcpy2D(obs, n * 5 * sizeof(double), c->d_trace + off * 5,
                           ne * 5 * sizeof(double), n * 5 * sizeof(double), rows,
                           cudaMemcpyDeviceToHost));
    if (rows > 0 && temp_of_rep)
        CK(c, cudaMemcpy2D(temp_of_rep, n * sizeof(int), c->d_trace_tor + off, ne * sizeof(int),
                           n * sizeof(int), rows, cudaMemcpyDeviceToHost));
    if (ncycles) *ncycles = (int64_t)rows;
    return J1J2C_OK;
}

int j1j2c_get_flip_counts(void* ctx, int32_t conf, int32_t* counts)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf) || !counts) return fail(c, J1J2C_EINVAL, "bad conf or null output");
    if (!c->d_flips) return fail(c, J1J2C_ESTATE, "flip counts are not enabled");
    const Group& grp = c->G[c->conf_group[conf]];
    const Geo& g = grp.g;
    const int nrep = grp.nrep, lc = conf - grp.conf0;
    std::vector<int> buf((size_t)nrep * grp.lat_stride);
    std::vector<uint8_t> occ((size_t)g.N);
    CK(c, cudaStreamSynchronize(c->st));
    CK(c, cudaMemcpy(buf.data(), c->d_flips + grp.spin_off + (size_t)lc * nrep * grp.lat_stride,
                     buf.size() * sizeof(int), cudaMemcpyDeviceToHost));
    CK(c, cudaMemcpy(occ.data(), c->d_occ + grp.mask_off + (size_t)lc * grp.lat_stride, g.N,
                     cudaMemcpyDeviceToHost));
    for (int sl = 0; sl < nrep; ++sl)
        for (int st = 0; st < g.N; ++st) {
            const int ci = compact_of_site(g, st);
            // Mark_vacancy_flipcounts (J:1168-1177): vacancies read -1
            counts[(size_t)sl * g.N + st] = occ[ci] ? buf[(size_t)sl * grp.lat_stride + ci] : -1;
        }
    return J1J2C_OK;
}

// Adds the sweep time of every cycle whose profiling pair is pending (waits for the last pair).
int drain_profile(Ctx* c)
{
    for (int k = 0; k < c->prof_pending; ++k) {
        CK(c, cudaEventSynchronize(c->pev1[k]));
        float ms = 0.0f;
        CK(c, cudaEventElapsedTime(&ms, c->pev0[k], c->pev1[k]));
        c->prof_ms += ms;
        c->prof_launches += 1;
        c->prof_attempts += c->occ_total * c->P.ptswapever;
    }
    c->prof_pending = 0;
    return J1J2C_OK;
}

// Reads the device error word and clears it (each give-up is reported once; the context stays
// usable).  Called after the stream has drained.
int take_device_error(Ctx* c, int& herr)
{
    herr = 0;
    CK(c, cudaMemcpy(&herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost));
    if (herr) {
        CK(c, cudaMemset(c->d_err, 0, sizeof(int)));
        // a level-free growth that gave up may have left list entries behind
        if (c->d_labels) CK(c, fill_labels(c));
    }
    return J1J2C_OK;
}

int j1j2c_enqueue(void* ctx, int32_t ncycles, int32_t measure, int32_t restart_swap_phase)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (ncycles < 0) return fail(c, J1J2C_EINVAL, "ncycles must be >= 0");
    for (int k = 0; k < c->nconf; ++k)
        if (!c->have_dis[k] || !c->have_ladder[k] || !c->have_spins[k])
            return fail(c, J1J2C_ESTATE,
                        "conf " + std::to_string(k) + " lacks disorder, ladder or spins");
    const int m = measure ? 1 : 0;
    if (restart_swap_phase) {
        c->host_ctl[1] = 1;
        CK(c, cudaMemcpyAsync(c->d_ctl + 1, &c->host_ctl[1], sizeof(uint32_t),
                              cudaMemcpyHostToDevice, c->st));
    }
    for (auto& grp : c->G) {
        int rct = autotune(c, grp);
        if (rct == J1J2C_OK && c->wolff && bits_of(c, grp)) rct = ensure_act(c);
        if (rct != J1J2C_OK) return rct;
    }
    {
        const int rct = tune_multi(c);
        if (rct != J1J2C_OK) return rct;
    }
    const bool direct = (c->P.flags & J1J2C_FLAG_NO_GRAPH) != 0;
    if (!direct && !c->graph[m]) {
        int rc = build_graph(c, m);
        if (rc != J1J2C_OK) return rc;
    }
    for (int k = 0; k < ncycles; ++k) {
        if (take_injected(2))
            return cuda_fail(c, cudaErrorLaunchFailure, "PT-cycle launch (injected failure)");
        cudaEvent_t e0 = c->ev0, e1 = c->ev1;
        if (c->profile) {
            if (c->prof_pending == kProfPool) {
                const int rc = drain_profile(c);
                if (rc != J1J2C_OK) return rc;
            }
            e0 = c->pev0[c->prof_pending];
            e1 = c->pev1[c->prof_pending];
            ++c->prof_pending;
        }
        if (direct) {
            CK(c, enqueue_cycle(c, m, c->st, e0, e1));
            continue;
        }
        if (c->profile) {
            CK(c, cudaGraphExecEventRecordNodeSetEvent(c->graph[m], c->graph_ev[m][0], e0));
            CK(c, cudaGraphExecEventRecordNodeSetEvent(c->graph[m], c->graph_ev[m][1], e1));
        }
        CK(c, cudaGraphLaunch(c->graph[m], c->st));
    }
    return J1J2C_OK;
}

int j1j2c_sync(void* ctx)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    CK(c, cudaStreamSynchronize(c->st));
    if (c->profile) {
        const int rc = drain_profile(c);
        if (rc != J1J2C_OK) return rc;
    }
    CK(c, cudaGetLastError());
    bool bounded = c->wolff;  // kernels whose bounded waits or retries report through d_err
    for (const Group& grp : c->G) bounded = bounded || grp.var.stream || grp.var.coop;
    if (bounded) {
        int herr = 0;
        const int rc = take_device_error(c, herr);
        if (rc != J1J2C_OK) return rc;
        if (herr)
            return fail(c, J1J2C_ETIMEOUT,
                        "a bounded device wait gave up (Wolff union-find retries, a wait of the "
                        "level-free Wolff growth, a bulk-copy wait of the streaming sweep kernel "
                        "or a grid barrier of the cooperative form)");
    }
    return J1J2C_OK;
}

int j1j2c_run(void* ctx, int32_t ncycles, int32_t measure, int32_t restart_swap_phase)
{
    const int rc = j1j2c_enqueue(ctx, ncycles, measure, restart_swap_phase);
    return rc != J1J2C_OK ? rc : j1j2c_sync(ctx);
}

int j1j2c_wolff(void* ctx, int64_t* cluster_sizes)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    for (int k = 0; k < c->nconf; ++k)
        if (!c->have_dis[k] || !c->have_ladder[k] || !c->have_spins[k])
            return fail(c, J1J2C_ESTATE, "every conf needs disorder, ladder and spins");
    CK(c, alloc_labels(c));
    for (auto& grp : c->G)
        if (bits_of(c, grp)) {
            const int rc = ensure_act(c);
            if (rc != J1J2C_OK) return rc;
        }
    for (auto& grp : c->G) CK(c, enqueue_wolff(c, grp, c->st));
    if (cluster_sizes)
        CK(c, cudaMemcpyAsync(cluster_sizes, c->d_csize, sizeof(long long) * c->nentries,
                              cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    int herr = 0;
    const int rc = take_device_error(c, herr);
    if (rc != J1J2C_OK) return rc;
    if (herr)
        return fail(c, J1J2C_ETIMEOUT,
                    "Wolff union-find exceeded its retry budget, or a wait of the level-free "
                    "growth gave up");
    return J1J2C_OK;
}

int j1j2c_inject_fault(int32_t kind)
{
    if (kind < 0 || kind > 2) return J1J2C_EINVAL;
    g_inject.store(kind);
    return J1J2C_OK;
}

int j1j2c_set_retry_budget(void* ctx, int32_t tries)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (tries < 0) return fail(c, J1J2C_EINVAL, "the retry budget must be >= 0");
    c->uf_tries = tries;
    free_graphs(c);  // captured graphs hold the old budget in their kernel arguments
    return J1J2C_OK;
}

int j1j2c_get_cluster_sizes(void* ctx, int32_t conf, int64_t* out)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (conf >= c->nconf || !out) return fail(c, J1J2C_EINVAL, "bad conf or null output");
    const size_t off = conf < 0 ? 0 : (size_t)c->conf_rbase[conf];
    const size_t nr = conf < 0 ? (size_t)c->nentries : (size_t)c->conf_nrep[conf];
    CK(c, cudaMemcpyAsync(out, c->d_csize + off, sizeof(long long) * nr, cudaMemcpyDeviceToHost,
                          c->st));
    CK(c, cudaStreamSynchronize(c->st));
    return J1J2C_OK;
}

int j1j2c_metro_sweep_fp64(void* ctx, int32_t conf, int32_t rep, double beta,
                           uint32_t sweep_index, int32_t nsweeps, double* mag, double* en,
                           double* strx, double* stry)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf) || rep < 0 || rep >= c->conf_nrep[conf])
        return fail(c, J1J2C_EINVAL, "conf or replica out of range");
    if (!c->have_dis[conf] || !c->have_spins[conf])
        return fail(c, J1J2C_ESTATE, "conf lacks disorder or spins");
    if (nsweeps < 0 || !std::isfinite(beta) || beta < 0.0)
        return fail(c, J1J2C_EINVAL, "bad nsweeps or beta");
    Group& grp = c->G[c->conf_group[conf]];
    SweepVariant v;
    size_t smem;
    int nt;
    int rc = choose_variant(c, grp, true, v, smem, nt);
    if (rc != J1J2C_OK) return rc;
    SweepArgs a = group_args(c, grp);
    const int lat = (conf - grp.conf0) * grp.nrep + rep;
    a.lat0 = lat;
    a.nsweeps = nsweeps;
    a.use_override = 1;
    a.beta_override = beta;
    a.sweep_override = sweep_index;
    CK(c, enqueue_group(c, grp, v, nt, smem, a, 1, c->st, false));
    LatObs o;
    CK(c, cudaMemcpyAsync(&o, a.obs + lat, sizeof o, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    const double dn = (double)c->nocc[conf];
    if (mag) *mag = (double)o.M / dn;
    if (en) *en = ((double)o.eacc * 0x1p-33) / dn;
    if (strx) *strx = (double)o.SX / dn;
    if (stry) *stry = (double)o.SY / dn;
    return J1J2C_OK;
}

int j1j2c_audit_fp32(void* ctx, int32_t nsweeps, int64_t* attempts, int64_t* mismatches)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (nsweeps < 0) return fail(c, J1J2C_EINVAL, "nsweeps must be >= 0");
    for (int k = 0; k < c->nconf; ++k)
        if (!c->have_dis[k] || !c->have_ladder[k] || !c->have_spins[k])
            return fail(c, J1J2C_ESTATE, "every conf needs disorder, ladder and spins");
    const size_t budget = smem_budget(c);
    CK(c, cudaMemsetAsync(c->d_audit, 0, 2 * sizeof(unsigned long long), c->st));
    for (auto& grp : c->G) {
        SweepVariant v{};
        v.fp64 = true;
        v.masks = c->masks;
        v.mode = kModeAudit;
        const size_t smem = sweep_smem_bytes(grp.g, v);
        if (smem > budget)
            return fail(c, J1J2C_EINVAL, "the audit needs lattices that fit shared memory");
        CK(c, prepare_sweep_variant(v, smem));
        int nt = ((grp.g.Nc + 31) / 32) * 32;
        if (nt > 512) nt = 512;
        if (nt < 64) nt = 64;
        SweepArgs a = group_args(c, grp);
        a.nsweeps = nsweeps;
        CK(c, launch_sweep(a, v, grp.nlat(), nt, smem, c->st));
    }
    unsigned long long h[2];
    CK(c, cudaMemcpyAsync(h, c->d_audit, sizeof h, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    if (attempts) *attempts += (int64_t)h[0];
    if (mismatches) *mismatches += (int64_t)h[1];
    return J1J2C_OK;
}

int j1j2c_get_slot_sums(void* ctx, int32_t conf, j1j2c_slot_sums* out)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (conf >= c->nconf || !out) return fail(c, J1J2C_EINVAL, "bad conf or null output");
    const size_t off = conf < 0 ? 0 : (size_t)c->conf_rbase[conf];
    const int nr = conf < 0 ? c->nentries : c->conf_nrep[conf];
    // straight into the caller's records (two strided copies; DMA when the buffer is pinned)
    CK(c, cudaMemcpy2DAsync(out, sizeof(j1j2c_slot_sums), c->d_sums + off * 22, 22 * sizeof(double),
                            22 * sizeof(double), (size_t)nr, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaMemcpy2DAsync(&out[0].nmeasure, sizeof(j1j2c_slot_sums), c->d_nmeas + off,
                            sizeof(long long), sizeof(long long), (size_t)nr,
                            cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    return J1J2C_OK;
}

int j1j2c_get_pt_stats(void* ctx, int32_t conf, int64_t* attempts, int64_t* accepts,
                       int32_t* visited_both)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    const size_t off = (size_t)c->conf_rbase[conf];
    const int nrep = c->conf_nrep[conf];
    std::vector<long long> at((size_t)nrep), ac((size_t)nrep);
    std::vector<uint8_t> vis((size_t)nrep);
    CK(c, cudaMemcpyAsync(at.data(), c->d_att + off, at.size() * 8, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaMemcpyAsync(ac.data(), c->d_acc + off, ac.size() * 8, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaMemcpyAsync(vis.data(), c->d_vis + off, vis.size(), cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    for (int k = 0; k + 1 < nrep; ++k) {
        if (attempts) attempts[k] = at[k];
        if (accepts) accepts[k] = ac[k];
    }
    if (visited_both) {
        int vb = 0;
        for (uint8_t v : vis) vb += (v == 3);
        *visited_both = vb;
    }
    return J1J2C_OK;
}

int j1j2c_get_maps(void* ctx, int32_t conf, int32_t* rep_at_temp, int32_t* temp_of_rep)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    const size_t off = (size_t)c->conf_rbase[conf], nb = sizeof(int) * c->conf_nrep[conf];
    if (rep_at_temp)
        CK(c, cudaMemcpyAsync(rep_at_temp, c->d_rat + off, nb, cudaMemcpyDeviceToHost, c->st));
    if (temp_of_rep)
        CK(c, cudaMemcpyAsync(temp_of_rep, c->d_tor + off, nb, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    return J1J2C_OK;
}

int j1j2c_get_spins(void* ctx, int32_t conf, int32_t rep, int8_t* out)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf) || rep < 0 || rep >= c->conf_nrep[conf] || !out)
        return fail(c, J1J2C_EINVAL, "bad conf, replica or output");
    const Group& grp = c->G[c->conf_group[conf]];
    const Geo& g = grp.g;
    std::vector<uint8_t> buf((size_t)g.N);
    const size_t lat = (size_t)(conf - grp.conf0) * grp.nrep + rep;
    CK(c, cudaMemcpyAsync(buf.data(), c->d_spins + grp.spin_off + lat * grp.lat_stride, g.N,
                          cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    for (int s = 0; s < g.N; ++s) out[s] = (int8_t)((int)buf[compact_of_site(g, s)] - 1);
    return J1J2C_OK;
}

int j1j2c_get_observables(void* ctx, int32_t conf, double* out)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (conf >= c->nconf || !out) return fail(c, J1J2C_EINVAL, "bad conf or null output");
    const size_t off = conf < 0 ? 0 : (size_t)c->conf_rbase[conf];
    const size_t nr = conf < 0 ? (size_t)c->nentries : (size_t)c->conf_nrep[conf];
    CK(c, cudaMemcpyAsync(out, c->d_last + off * 5, sizeof(double) * 5 * nr,
                          cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    return J1J2C_OK;
}

int j1j2c_enumerate_exact(int32_t L, int32_t H, double J1h, double J1v, double J2, double J3,
                          const double* p, const int8_t* occu, const int8_t* jh,
                          const int8_t* jv, int32_t nbeta, const double* beta, double* out)
{
    g_create_error.clear();
    const int N = L * H * L;
    if (L < 2 || H < 2 || (L & 1) || (H & 1) || N > 32 || !p || !beta || !out || nbeta < 1 ||
        nbeta > kEnumBeta) {
        g_create_error = "enumeration needs even L, H with L*L*H <= 32 and 1..4 betas";
        return J1J2C_EINVAL;
    }
    EnumArgs a{};
    a.N = N;
    a.LB = N < 16 ? N : 16;
    a.J1h = J1h;
    a.J1v = J1v;
    a.J2 = J2;
    a.J3 = J3;
    a.nbeta = nbeta;
    double pmax = 0.0;
    int nocc = 0;
    for (int i = 0; i < N; ++i) {
        const int x = i % L, y = (i / L) % L, z = i / (L * L);
        auto site = [&](int dx, int dy, int dz) {
            return ((x + dx + L) % L) + L * ((y + dy + L) % L) + L * L * ((z + dz + H) % H);
        };
        const int nb[10] = {site(0, 1, 0),  site(0, -1, 0), site(1, 0, 0),  site(-1, 0, 0),
                            site(1, 1, 0),  site(-1, 1, 0), site(1, -1, 0), site(-1, -1, 0),
                            site(0, 0, 1),  site(0, 0, -1)};
        for (int k = 0; k < 10; ++k) a.nbr[i][k] = (int8_t)nb[k];
        a.p[i] = p[i];
        a.occ[i] = occu ? (occu[i] != 0) : 1;
        a.jh[i] = jh ? (jh[i] != 0) : 1;
        a.jv[i] = jv ? (jv[i] != 0) : 1;
        a.px[i] = (uint8_t)(x & 1);
        a.py[i] = (uint8_t)(y & 1);
        nocc += a.occ[i];
        pmax = std::fmax(pmax, std::fabs(p[i]));
        if (!std::isfinite(p[i])) {
            g_create_error = "p must be finite";
            return J1J2C_EINVAL;
        }
    }
    if (nocc == 0) {
        g_create_error = "no occupied site";
        return J1J2C_EINVAL;
    }
    a.nocc = (double)nocc;
    a.E0 = -0.5 * N *
           (2 * std::fabs(J1h) + 2 * std::fabs(J1v) + 4 * std::fabs(J2) + 2 * std::fabs(J3) +
            8 * pmax) - 1.0;
    for (int b = 0; b < nbeta; ++b) {
        if (!std::isfinite(beta[b]) || beta[b] < 0.0) {
            g_create_error = "beta must be finite and >= 0";
            return J1J2C_EINVAL;
        }
        a.beta[b] = beta[b];
    }
    const int nb = enum_blocks(a);
    const size_t np = (size_t)nb * kEnumBeta * kEnumSums;
    double* d_part = nullptr;  // scratch: one partial-sum record per block
    cudaError_t e = dev_malloc(&d_part, np * sizeof(double));
    if (e != cudaSuccess) {
        g_create_error = std::string("enumeration scratch: ") + cudaGetErrorString(e);
        return J1J2C_ENOMEM;
    }
    std::vector<double> part(np);
    e = launch_enumerate(a, d_part, 0);
    if (e == cudaSuccess) e = cudaMemcpy(part.data(), d_part, np * sizeof(double),
                                         cudaMemcpyDeviceToHost);
    cudaFree(d_part);
    if (e != cudaSuccess) {
        g_create_error = std::string("enumeration: ") + cudaGetErrorString(e);
        return J1J2C_ECUDA;
    }
    for (int b = 0; b < nbeta; ++b) {
        double s[kEnumSums] = {0};
        for (int blk = 0; blk < nb; ++blk)
            for (int q = 0; q < kEnumSums; ++q)
                s[q] += part[((size_t)blk * kEnumBeta + b) * kEnumSums + q];
        double* o = out + (size_t)b * kEnumSums;
        o[0] = std::log(s[0]) - beta[b] * a.E0;  // ln Z
        for (int q = 1; q < kEnumSums; ++q) o[q] = s[q] / s[0];
    }
    return J1J2C_OK;
}

int j1j2c_get_profile(void* ctx, double* sweep_ms, int64_t* launches, int64_t* attempts)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (sweep_ms) *sweep_ms = c->prof_ms;
    if (launches) *launches = c->prof_launches;
    if (attempts) *attempts = c->prof_attempts;
    return J1J2C_OK;
}

int j1j2c_get_config(void* ctx, int32_t* block_threads, int32_t* sites_per_thread,
                     int32_t* smem_bytes)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (c->multi && multi_possible(c)) {  // the persistent launch over every group
        if (block_threads) *block_threads = multi_threads();
        if (sites_per_thread) *sites_per_thread = 4;
        if (smem_bytes) *smem_bytes = (int32_t)multi_smem_bytes();
        return J1J2C_OK;
    }
    const Group& grp = c->G[0];
    if (block_threads) *block_threads = grp.nthreads;
    if (sites_per_thread) *sites_per_thread = grp.var.quad ? 4 : 1;
    if (smem_bytes) *smem_bytes = (int32_t)grp.smem;
    return J1J2C_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// Checkpoint / resume: the whole device state of a context as one host byte blob
// ------------------------------------------------------------------------------------------------
namespace {

struct StateHeader {
    char magic[8];
    uint32_t version, ngroups;
    int32_t nconf, nentries, precision, ptswapever;
    uint32_t seed, conf_base;
    double J1h, J1v, J2, J3;
    int64_t spin_bytes, p_elems, mask_bytes;
    uint32_t cycle, phase;
    j1j2c_diagnostics diag;
};
constexpr char kStateMagic[8] = {'J', '1', 'J', '2', 'C', 'S', 'T', '1'};

// Walks the sections of the blob in a fixed order; mode 0 counts, 1 saves (device -> blob),
// 2 loads (blob -> device).
struct StateIO {
    int mode;
    uint8_t* buf;
    size_t off = 0;
    cudaError_t err = cudaSuccess;
    void dev(void* d, size_t bytes)
    {
        if (mode == 1 && err == cudaSuccess && bytes)
            err = cudaMemcpy(buf + off, d, bytes, cudaMemcpyDeviceToHost);
        if (mode == 2 && err == cudaSuccess && bytes)
            err = cudaMemcpy(d, buf + off, bytes, cudaMemcpyHostToDevice);
        off += bytes;
    }
    void host(void* h, size_t bytes)
    {
        if (mode == 1 && bytes) std::memcpy(buf + off, h, bytes);
        if (mode == 2 && bytes) std::memcpy(h, buf + off, bytes);
        off += bytes;
    }
};

void state_sections(Ctx* c, StateIO& io)
{
    const size_t ne = (size_t)c->nentries, nc = (size_t)c->nconf;
    io.dev(c->d_spins, (size_t)c->spin_bytes);
    io.dev(c->d_pf, (size_t)c->p_elems * sizeof(float));
    io.dev(c->d_pd, (size_t)c->p_elems * sizeof(double));
    io.dev(c->d_bm, (size_t)c->mask_bytes);
    io.dev(c->d_occ, (size_t)c->mask_bytes);
    io.dev(c->d_nocc, nc * sizeof(int));
    io.dev(c->d_beta, ne * sizeof(double));
    io.dev(c->d_rat, ne * sizeof(int));
    io.dev(c->d_tor, ne * sizeof(int));
    io.dev(c->d_obs, ne * sizeof(LatObs));
    io.dev(c->d_sums, ne * 22 * sizeof(double));
    io.dev(c->d_nmeas, ne * sizeof(long long));
    io.dev(c->d_att, ne * sizeof(long long));
    io.dev(c->d_acc, ne * sizeof(long long));
    io.dev(c->d_vis, ne);
    io.dev(c->d_last, ne * 5 * sizeof(double));
    io.dev(c->d_csize, ne * sizeof(long long));
    io.host(c->have_dis.data(), nc);
    io.host(c->have_ladder.data(), nc);
    io.host(c->have_spins.data(), nc);
    io.host(c->nocc.data(), nc * sizeof(int));
    io.host(c->conf_masks.data(), nc * sizeof(int));
    io.host(c->conf_vac.data(), nc * sizeof(int));
    if (c->d_loc_s) {
        io.dev(c->d_loc_s, (size_t)c->mask_bytes * sizeof(int));
        io.dev(c->d_loc_n, (size_t)c->mask_bytes * sizeof(int));
        io.dev(c->d_loc_samples, nc * sizeof(long long));
    }
    if (c->d_hist) {
        io.dev(c->d_hist, ne * (size_t)c->diag.hist_bins * sizeof(long long));
        io.dev(c->d_hist_lo, ne * sizeof(double));
        io.dev(c->d_hist_bs, ne * sizeof(double));
    }
    if (c->d_trace) {
        io.dev(c->d_trace, (size_t)c->diag.trace_cycles * ne * 5 * sizeof(double));
        io.dev(c->d_trace_tor, (size_t)c->diag.trace_cycles * ne * sizeof(int));
    }
    if (c->d_flips) io.dev(c->d_flips, (size_t)c->spin_bytes * sizeof(int));
}

StateHeader make_header(Ctx* c)
{
    StateHeader h{};
    std::memcpy(h.magic, kStateMagic, 8);
    h.version = 1;
    h.ngroups = (uint32_t)c->G.size();
    h.nconf = c->nconf;
    h.nentries = c->nentries;
    h.precision = c->P.precision;
    h.ptswapever = c->P.ptswapever;
    h.seed = c->P.seed;
    h.conf_base = c->P.conf_base;
    h.J1h = c->P.J1h;
    h.J1v = c->P.J1v;
    h.J2 = c->P.J2;
    h.J3 = c->P.J3;
    h.spin_bytes = c->spin_bytes;
    h.p_elems = c->p_elems;
    h.mask_bytes = c->mask_bytes;
    h.cycle = c->host_ctl[0];
    h.phase = c->host_ctl[1];
    h.diag = c->diag;
    return h;
}

size_t state_bytes(Ctx* c)
{
    StateIO io{0, nullptr};
    state_sections(c, io);
    return sizeof(StateHeader) + c->G.size() * 4 * sizeof(int32_t) + io.off;
}

}  // namespace

extern "C" {

int j1j2c_state_size(void* ctx, int64_t* bytes)
{
    if (!ctx || !bytes) return J1J2C_EINVAL;
    *bytes = (int64_t)state_bytes(static_cast<Ctx*>(ctx));
    return J1J2C_OK;
}

int j1j2c_save_state(void* ctx, void* buf, int64_t size)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!buf || size < (int64_t)state_bytes(c))
        return fail(c, J1J2C_EINVAL, "state buffer missing or smaller than j1j2c_state_size");
    CK(c, cudaStreamSynchronize(c->st));
    CK(c, cudaMemcpy(c->host_ctl, c->d_ctl, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    uint8_t* b = static_cast<uint8_t*>(buf);
    StateHeader h = make_header(c);
    std::memcpy(b, &h, sizeof h);
    size_t off = sizeof h;
    for (const Group& grp : c->G) {
        const int32_t shape[4] = {grp.g.L, grp.g.H, grp.nconf, grp.nrep};
        std::memcpy(b + off, shape, sizeof shape);
        off += sizeof shape;
    }
    StateIO io{1, b + off};
    state_sections(c, io);
    if (io.err != cudaSuccess) return cuda_fail(c, io.err, "saving the state");
    return J1J2C_OK;
}

int j1j2c_load_state(void* ctx, const void* buf, int64_t size)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!buf || size < (int64_t)sizeof(StateHeader)) return fail(c, J1J2C_EINVAL, "state blob too small");
    const uint8_t* b = static_cast<const uint8_t*>(buf);
    StateHeader h;
    std::memcpy(&h, b, sizeof h);
    const StateHeader mine = make_header(c);
    if (std::memcmp(h.magic, kStateMagic, 8) != 0 || h.version != 1)
        return fail(c, J1J2C_EINVAL, "not a libj1j2cuda state blob");
    if (h.ngroups != mine.ngroups || h.nconf != mine.nconf || h.nentries != mine.nentries ||
        h.precision != mine.precision || h.ptswapever != mine.ptswapever || h.seed != mine.seed ||
        h.conf_base != mine.conf_base || h.J1h != mine.J1h || h.J1v != mine.J1v ||
        h.J2 != mine.J2 || h.J3 != mine.J3 || h.spin_bytes != mine.spin_bytes)
        return fail(c, J1J2C_EINVAL, "state blob from a context with other parameters");
    size_t off = sizeof h;
    for (const Group& grp : c->G) {
        int32_t shape[4];
        std::memcpy(shape, b + off, sizeof shape);
        off += sizeof shape;
        if (shape[0] != grp.g.L || shape[1] != grp.g.H || shape[2] != grp.nconf ||
            shape[3] != grp.nrep)
            return fail(c, J1J2C_EINVAL, "state blob from a context with other lattice shapes");
    }
    // the blob's diagnostics decide which optional buffers exist
    int rc = j1j2c_set_diagnostics(ctx, &h.diag);
    if (rc != J1J2C_OK) return rc;
    if (size < (int64_t)state_bytes(c)) return fail(c, J1J2C_EINVAL, "state blob truncated");
    CK(c, cudaStreamSynchronize(c->st));
    StateIO io{2, const_cast<uint8_t*>(b) + off};
    state_sections(c, io);
    if (io.err != cudaSuccess) return cuda_fail(c, io.err, "loading the state");
    c->host_ctl[0] = h.cycle;
    c->host_ctl[1] = h.phase;
    c->host_ctl[2] = 0;
    CK(c, cudaMemcpy(c->d_ctl, c->host_ctl, 4 * sizeof(uint32_t), cudaMemcpyHostToDevice));
    {  // the acceptance scales follow the restored ladder
        std::vector<double> beta((size_t)c->nentries);
        CK(c, cudaMemcpy(beta.data(), c->d_beta, sizeof(double) * beta.size(),
                         cudaMemcpyDeviceToHost));
        const std::vector<float> kb = acceptance_scales(beta.data(), c->nentries);
        CK(c, cudaMemcpy(c->d_kb, kb.data(), sizeof(float) * kb.size(), cudaMemcpyHostToDevice));
    }
    bool masks = false, vac = false;
    for (int k : c->conf_masks) masks = masks || k;
    for (int k : c->conf_vac) vac = vac || k;
    free_graphs(c);
    c->masks = masks;
    c->vac = vac;
    for (auto& gr : c->G) {
        rc = choose_variant(c, gr, c->P.precision == J1J2C_FP64_PLAIN, gr.var, gr.smem,
                            gr.nthreads);
        if (rc != J1J2C_OK) return rc;
        gr.tuned = false;
    }
    c->occ_total = 0;
    for (int k = 0; k < c->nconf; ++k) c->occ_total += (long long)c->nocc[k] * c->conf_nrep[k];
    return J1J2C_OK;
}

}  // extern "C"
