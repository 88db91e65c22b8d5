// C-ABI of libj1j2cuda: context management, layout conversion between the reference's site order
// and the engine's colour-compact layout, the CUDA-graph replay of one PT cycle, and the outputs.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
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

struct Ctx {
    j1j2c_params P{};
    Geo g{};
    int nconf = 0, nrep = 0, nlat = 0;
    long long lat_stride = 0, p_stride = 0;

    uint8_t* d_spins = nullptr;
    float* d_pf = nullptr;
    double* d_pd = nullptr;
    uint8_t* d_bm = nullptr;
    uint8_t* d_occ = nullptr;
    double* d_beta = nullptr;
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
    unsigned long long* d_audit = nullptr;

    std::vector<uint8_t> have_dis, have_ladder, have_spins;
    std::vector<int> nocc;
    std::vector<uint8_t> bm_host;  // per conf, compact; tells whether bond masks are present
    std::vector<int> conf_masks;
    bool masks = false;

    cudaStream_t own = nullptr, st = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    SweepVariant var{};
    int nthreads = 0;
    size_t smem = 0;
    long long occ_total = 0;

    bool tuned = false;
    bool profile = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double prof_ms = 0.0;
    long long prof_launches = 0, prof_attempts = 0;

    uint32_t host_ctl[2] = {0, 1};
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
    return fail(c, J1J2C_ECUDA, m);
}

#define CK(c, call)                                               \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail((c), e_, #call); \
    } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t n)
{
    return cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T) + 16);
}

void free_graphs(Ctx* c)
{
    for (auto& gx : c->graph)
        if (gx) {
            cudaGraphExecDestroy(gx);
            gx = nullptr;
        }
}

void release(Ctx* c)
{
    free_graphs(c);
    void* ptrs[] = {c->d_spins, c->d_pf,   c->d_pd,   c->d_bm,  c->d_occ,   c->d_beta,
                    c->d_rat,   c->d_tor,  c->d_obs,  c->d_sums, c->d_nmeas, c->d_att,
                    c->d_acc,   c->d_vis,  c->d_last, c->d_ctl, c->d_nocc,  c->d_audit};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own) cudaStreamDestroy(c->own);
}

size_t smem_budget(Ctx* c)
{
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->P.device) !=
        cudaSuccess)
        return 0;
    return (size_t)optin - 2048;  // static shared memory of the reduction
}

// Kernel shape for the context's lattices: the shape-specialised kernel when one exists for
// (precision, L, H) and no bond is diluted (its CTA size autotuned at the first run unless
// block_threads names one), else the generic quad path when L/2 is a multiple of 4, else the
// per-site path; the random field is staged in shared memory when it fits next to the spins.
int choose_variant(Ctx* c, bool fp64, SweepVariant& v, size_t& smem, int& nthreads)
{
    const size_t budget = smem_budget(c);
    if (budget == 0) return fail(c, J1J2C_ECUDA, "cannot query the shared-memory limit");
    v = SweepVariant{};
    v.fp64 = fp64;
    v.masks = c->masks;
    v.mode = kModeSweep;
    if (!(c->P.flags & (J1J2C_FLAG_GENERIC | J1J2C_FLAG_NO_FIXED))) {
        int nts[8];
        bool sp[8];
        const int n = fixed_candidates(fp64, c->g.L, c->g.H, c->masks, nts, sp, 8);
        int pick = n > 0 ? 0 : -1;
        for (int k = 0; k < n; ++k)
            if (nts[k] == c->P.block_threads) pick = k;
        if (pick >= 0) {
            v.fixed_nt = nts[pick];
            v.quad = true;
            v.stage_p = sp[pick];
            smem = sweep_smem_bytes(c->g, v);
            if (smem <= budget) {
                nthreads = nts[pick];
                SweepArgs none{};
                none.g = c->g;
                CK(c, launch_fixed(none, fp64, nthreads, 0, smem, nullptr, true));
                return J1J2C_OK;
            }
            v.fixed_nt = 0;
        }
    }
    v.quad = (c->g.Lh % 4 == 0) && !(c->P.flags & J1J2C_FLAG_GENERIC);
    v.stage_p = true;
    smem = sweep_smem_bytes(c->g, v);
    if (smem > budget) {
        v.stage_p = false;
        smem = sweep_smem_bytes(c->g, v);
    }
    if (smem > budget)
        return fail(c, J1J2C_EINVAL,
                    "lattice of " + std::to_string(c->g.N) +
                        " sites does not fit the shared-memory sweep kernel");
    const int work = v.quad ? c->g.Nc / 4 : c->g.Nc;
    if (c->P.block_threads > 0) {
        nthreads = c->P.block_threads;
    } else {
        nthreads = ((work + 31) / 32) * 32;
        if (nthreads > 1024) nthreads = 1024;
        if (nthreads < 64) nthreads = 64;
    }
    CK(c, prepare_sweep_variant(v, smem));
    return J1J2C_OK;
}

SweepArgs base_args(Ctx* c)
{
    SweepArgs a{};
    a.g = c->g;
    a.spins = c->d_spins;
    a.lat_stride = c->lat_stride;
    a.pf = c->d_pf;
    a.pd = c->d_pd;
    a.bm = c->masks ? c->d_bm : nullptr;
    a.p_stride = c->p_stride;
    a.beta = c->d_beta;
    a.temp_of_rep = c->d_tor;
    a.ctl = c->d_ctl;
    a.obs = c->d_obs;
    a.audit = c->d_audit;
    a.J1h = c->P.J1h;
    a.J1v = c->P.J1v;
    a.J2 = c->P.J2;
    a.J3 = c->P.J3;
    a.J1hf = (float)c->P.J1h;
    a.J1vf = (float)c->P.J1v;
    a.J2f = (float)c->P.J2;
    a.J3f = (float)c->P.J3;
    a.nrep = c->nrep;
    a.nsweeps = c->P.ptswapever;
    a.ptswapever = c->P.ptswapever;
    a.seed = c->P.seed;
    a.conf_base = c->P.conf_base;
    a.lat0 = 0;
    a.use_override = 0;
    return a;
}

SwapArgs swap_args(Ctx* c, int measure)
{
    SwapArgs s{};
    s.obs = c->d_obs;
    s.beta = c->d_beta;
    s.nocc = c->d_nocc;
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
    s.nrep = c->nrep;
    s.measure = measure;
    s.seed = c->P.seed;
    s.conf_base = c->P.conf_base;
    return s;
}

// one PT cycle: fused sweeps + observables of every lattice, then swap / accumulate
cudaError_t enqueue_cycle(Ctx* c, int measure, cudaStream_t st)
{
    SweepArgs a = base_args(c);
    cudaError_t e;
    if (c->profile && (e = cudaEventRecordWithFlags(c->ev0, st, cudaEventRecordExternal)) !=
                           cudaSuccess)
        return e;
    if ((e = launch_sweep(a, c->var, c->nlat, c->nthreads, c->smem, st)) != cudaSuccess) return e;
    if (c->profile && (e = cudaEventRecordWithFlags(c->ev1, st, cudaEventRecordExternal)) !=
                           cudaSuccess)
        return e;
    return launch_swap(swap_args(c, measure), st);
}

int build_graph(Ctx* c, int measure)
{
    cudaGraph_t graph = nullptr;
    CK(c, cudaStreamBeginCapture(c->own, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = enqueue_cycle(c, measure, c->own);
    cudaError_t e2 = cudaStreamEndCapture(c->own, &graph);
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(c, e, "capturing the PT-cycle graph");
    }
    if (e2 != cudaSuccess) return cuda_fail(c, e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->graph[measure], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
    return J1J2C_OK;
}

bool valid_conf(Ctx* c, int conf) { return conf >= 0 && conf < c->nconf; }

// Autotuner: times every CTA size of the shape-specialised kernel on a scratch copy of the
// context's lattices (the live state is not touched) and keeps the fastest.  Choices are cached
// per (precision, L, H, lattice count) for the life of the process.
std::mutex g_tune_mu;
std::map<std::tuple<bool, int, int, int>, int> g_tune_cache;

int autotune(Ctx* c)
{
    if (c->tuned) return J1J2C_OK;
    c->tuned = true;
    if (c->var.fixed_nt == 0 || c->P.block_threads > 0) return J1J2C_OK;
    int nts[8];
    bool sp[8];
    const int n = fixed_candidates(c->var.fp64, c->g.L, c->g.H, c->masks, nts, sp, 8);
    if (n <= 1) return J1J2C_OK;
    const auto key = std::make_tuple(c->var.fp64, c->g.L, c->g.H, c->nlat);
    int best_nt = 0;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) best_nt = it->second;
    }
    const size_t budget = smem_budget(c);
    if (best_nt == 0) {
        uint8_t* tmp = nullptr;
        LatObs* tobs = nullptr;
        const size_t bytes = (size_t)c->nlat * c->lat_stride;
        CK(c, cudaMalloc(&tmp, bytes));
        if (cudaMalloc(&tobs, sizeof(LatObs) * c->nlat) != cudaSuccess) {
            cudaFree(tmp);
            return fail(c, J1J2C_ENOMEM, "autotuner scratch");
        }
        cudaError_t e = cudaMemcpyAsync(tmp, c->d_spins, bytes, cudaMemcpyDeviceToDevice, c->own);
        SweepArgs a = base_args(c);
        a.spins = tmp;
        a.obs = tobs;
        a.use_override = 1;
        a.beta_override = 1.0 / 9.5;
        a.sweep_override = 0x5EED0000u;
        float best_ms = 1e30f;
        for (int k = 0; k < n && e == cudaSuccess; ++k) {
            SweepVariant v = c->var;
            v.fixed_nt = nts[k];
            v.stage_p = sp[k];
            const size_t sm = sweep_smem_bytes(c->g, v);
            if (sm > budget) continue;
            if ((e = launch_fixed(a, v.fp64, nts[k], 0, sm, nullptr, true)) != cudaSuccess) break;
            if ((e = launch_fixed(a, v.fp64, nts[k], c->nlat, sm, c->own, false)) != cudaSuccess)
                break;
            cudaEventRecord(c->ev0, c->own);
            for (int r = 0; r < 3 && e == cudaSuccess; ++r)
                e = launch_fixed(a, v.fp64, nts[k], c->nlat, sm, c->own, false);
            cudaEventRecord(c->ev1, c->own);
            if (e == cudaSuccess) e = cudaEventSynchronize(c->ev1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            if (e == cudaSuccess && ms < best_ms) {
                best_ms = ms;
                best_nt = nts[k];
            }
        }
        cudaStreamSynchronize(c->own);
        cudaFree(tmp);
        cudaFree(tobs);
        if (e != cudaSuccess) return cuda_fail(c, e, "autotuning the sweep kernel");
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best_nt;
    }
    for (int k = 0; k < n; ++k)
        if (nts[k] == best_nt) {
            c->var.fixed_nt = nts[k];
            c->var.stage_p = sp[k];
            c->smem = sweep_smem_bytes(c->g, c->var);
            c->nthreads = nts[k];
            SweepArgs none{};
            none.g = c->g;
            CK(c, launch_fixed(none, c->var.fp64, c->nthreads, 0, c->smem, nullptr, true));
        }
    free_graphs(c);
    return J1J2C_OK;
}

}  // namespace

extern "C" {

const char* j1j2c_version(void) { return "j1j2cuda 0.1 (sm_103a)"; }

const char* j1j2c_last_error(void* ctx)
{
    if (!ctx) return g_create_error.c_str();
    return static_cast<Ctx*>(ctx)->err.c_str();
}

int j1j2c_create(void** out, const j1j2c_params* p)
{
    g_create_error.clear();
    if (!out || !p) {
        g_create_error = "null argument";
        return J1J2C_EINVAL;
    }
    *out = nullptr;
    auto bad = [](const std::string& m) {
        g_create_error = m;
        return J1J2C_EINVAL;
    };
    if (p->L < 2 || p->H < 2 || (p->L & 1) || (p->H & 1))
        return bad("L and H must be even and >= 2 (8-colour update)");
    if ((long long)p->L * p->L * p->H > (1ll << 28)) return bad("lattice too large");
    if (p->nconf < 1 || p->nreplica < 1) return bad("nconf and nreplica must be >= 1");
    if (p->ptswapever < 1) return bad("ptswapever must be positive (J:909-912)");
    if (p->precision != J1J2C_FP64_PLAIN && p->precision != J1J2C_FP32_BATCHED)
        return bad("precision must be J1J2C_FP64_PLAIN or J1J2C_FP32_BATCHED");
    if (p->block_threads < 0 || p->block_threads > 1024 || (p->block_threads % 32))
        return bad("block_threads must be 0 or a multiple of 32 up to 1024");
    if (!std::isfinite(p->J1h) || !std::isfinite(p->J1v) || !std::isfinite(p->J2) ||
        !std::isfinite(p->J3))
        return bad("couplings must be finite");

    Ctx* c = new Ctx();
    c->P = *p;
    c->g.L = p->L;
    c->g.H = p->H;
    c->g.Lh = p->L / 2;
    c->g.Hh = p->H / 2;
    c->g.N = p->L * p->L * p->H;
    c->g.Nc = c->g.Lh * c->g.Lh * c->g.Hh;
    c->g.Qr = (c->g.Lh + 3) / 4;
    c->nconf = p->nconf;
    c->nrep = p->nreplica;
    c->nlat = p->nconf * p->nreplica;
    c->lat_stride = ((long long)c->g.N + 15) & ~15ll;
    c->p_stride = ((long long)c->g.N + 3) & ~3ll;
    c->have_dis.assign(c->nconf, 0);
    c->have_ladder.assign(c->nconf, 0);
    c->have_spins.assign(c->nconf, 0);
    c->nocc.assign(c->nconf, 0);
    c->conf_masks.assign(c->nconf, 0);
    c->profile = (p->flags & J1J2C_FLAG_PROFILE) != 0;

    auto cfail = [&](cudaError_t e, const char* what) {
        g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
        release(c);
        delete c;
        return e == cudaErrorMemoryAllocation ? J1J2C_ENOMEM : J1J2C_ECUDA;
    };
    cudaError_t e = cudaSetDevice(p->device);
    if (e != cudaSuccess) return cfail(e, "cudaSetDevice");
    const size_t nl = (size_t)c->nlat, nc = (size_t)c->nconf;
    if ((e = dalloc(&c->d_spins, nl * c->lat_stride)) != cudaSuccess) return cfail(e, "spins");
    if ((e = dalloc(&c->d_pf, nc * c->p_stride)) != cudaSuccess) return cfail(e, "field");
    if ((e = dalloc(&c->d_pd, nc * c->p_stride)) != cudaSuccess) return cfail(e, "field");
    if ((e = dalloc(&c->d_bm, nc * c->lat_stride)) != cudaSuccess) return cfail(e, "masks");
    if ((e = dalloc(&c->d_occ, nc * c->lat_stride)) != cudaSuccess) return cfail(e, "occ");
    if ((e = dalloc(&c->d_beta, nl)) != cudaSuccess) return cfail(e, "beta");
    if ((e = dalloc(&c->d_rat, nl)) != cudaSuccess) return cfail(e, "maps");
    if ((e = dalloc(&c->d_tor, nl)) != cudaSuccess) return cfail(e, "maps");
    if ((e = dalloc(&c->d_obs, nl)) != cudaSuccess) return cfail(e, "obs");
    if ((e = dalloc(&c->d_sums, nl * 22)) != cudaSuccess) return cfail(e, "sums");
    if ((e = dalloc(&c->d_nmeas, nl)) != cudaSuccess) return cfail(e, "sums");
    if ((e = dalloc(&c->d_att, nl)) != cudaSuccess) return cfail(e, "pt stats");
    if ((e = dalloc(&c->d_acc, nl)) != cudaSuccess) return cfail(e, "pt stats");
    if ((e = dalloc(&c->d_vis, nl)) != cudaSuccess) return cfail(e, "pt stats");
    if ((e = dalloc(&c->d_last, nl * 5)) != cudaSuccess) return cfail(e, "obs");
    if ((e = dalloc(&c->d_ctl, 4)) != cudaSuccess) return cfail(e, "ctl");
    if ((e = dalloc(&c->d_nocc, nc)) != cudaSuccess) return cfail(e, "nocc");
    if ((e = dalloc(&c->d_audit, 2)) != cudaSuccess) return cfail(e, "audit");
    if ((e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking)) != cudaSuccess)
        return cfail(e, "stream");
    c->st = c->own;
    if ((e = cudaEventCreate(&c->ev0)) != cudaSuccess) return cfail(e, "event");
    if ((e = cudaEventCreate(&c->ev1)) != cudaSuccess) return cfail(e, "event");
    if ((e = cudaMemset(c->d_spins, 1, nl * c->lat_stride)) != cudaSuccess)
        return cfail(e, "memset");
    if ((e = cudaMemset(c->d_bm, 3, nc * c->lat_stride)) != cudaSuccess) return cfail(e, "memset");
    if ((e = cudaMemset(c->d_obs, 0, nl * sizeof(LatObs))) != cudaSuccess)
        return cfail(e, "memset");
    if ((e = cudaMemcpy(c->d_ctl, c->host_ctl, 2 * sizeof(uint32_t), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
        return cfail(e, "ctl");
    int rc = choose_variant(c, p->precision == J1J2C_FP64_PLAIN, c->var, c->smem, c->nthreads);
    if (rc != J1J2C_OK) {
        g_create_error = c->err;
        release(c);
        delete c;
        return rc;
    }
    *out = c;
    rc = j1j2c_reset_measurements(c, -1);
    if (rc != J1J2C_OK) {
        g_create_error = c->err;
        release(c);
        delete c;
        *out = nullptr;
        return rc;
    }
    return J1J2C_OK;
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

int j1j2c_set_disorder(void* ctx, int32_t conf, const double* p, const int8_t* occu,
                       const int8_t* jh, const int8_t* jv)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    if (!p) return fail(c, J1J2C_EINVAL, "p is null");
    const Geo& g = c->g;
    std::vector<double> pd((size_t)c->p_stride, 0.0);
    std::vector<float> pf((size_t)c->p_stride, 0.0f);
    std::vector<uint8_t> occ((size_t)c->lat_stride, 0), bm((size_t)c->lat_stride, 3);
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
    const size_t off = (size_t)conf;
    CK(c, cudaMemcpy(c->d_pd + off * c->p_stride, pd.data(), pd.size() * 8, cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_pf + off * c->p_stride, pf.data(), pf.size() * 4, cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_occ + off * c->lat_stride, occ.data(), occ.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_bm + off * c->lat_stride, bm.data(), bm.size(), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(c->d_nocc + conf, &nocc, sizeof(int), cudaMemcpyHostToDevice));
    c->nocc[conf] = nocc;
    c->conf_masks[conf] = anymask;
    bool masks = false;
    for (int k : c->conf_masks) masks = masks || k;
    if (masks != c->masks) {
        c->masks = masks;
        free_graphs(c);
        int rc = choose_variant(c, c->P.precision == J1J2C_FP64_PLAIN, c->var, c->smem,
                                c->nthreads);
        if (rc != J1J2C_OK) return rc;
        c->tuned = false;
    }
    c->have_dis[conf] = 1;
    c->have_spins[conf] = 0;  // vacancies changed: spins must be initialised again
    c->occ_total = 0;
    for (int k = 0; k < c->nconf; ++k) c->occ_total += (long long)c->nocc[k] * c->nrep;
    return J1J2C_OK;
}

int j1j2c_set_ladder(void* ctx, int32_t conf, const double* beta)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (conf >= c->nconf) return fail(c, J1J2C_EINVAL, "conf out of range");
    if (!beta) return fail(c, J1J2C_EINVAL, "beta is null");
    const int c0 = conf < 0 ? 0 : conf, nc = conf < 0 ? c->nconf : 1;
    for (int k = 0; k < nc * c->nrep; ++k)
        if (!std::isfinite(beta[k]) || beta[k] < 0.0)
            return fail(c, J1J2C_EINVAL, "beta must be finite and >= 0");
    CK(c, cudaMemcpyAsync(c->d_beta + (size_t)c0 * c->nrep, beta,
                          sizeof(double) * c->nrep * nc, cudaMemcpyHostToDevice, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    for (int k = c0; k < c0 + nc; ++k) c->have_ladder[k] = 1;
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
    const Geo& g = c->g;
    uint8_t* dst = c->d_spins + (size_t)conf * c->nrep * c->lat_stride;
    if (spins) {
        std::vector<uint8_t> occ((size_t)g.N);
        CK(c, cudaMemcpy(occ.data(), c->d_occ + (size_t)conf * c->lat_stride, g.N,
                         cudaMemcpyDeviceToHost));
        std::vector<uint8_t> buf((size_t)c->nrep * c->lat_stride, 1);
        for (int r = 0; r < c->nrep; ++r)
            for (int s = 0; s < g.N; ++s) {
                const int8_t v = spins[(size_t)r * g.N + s];
                if (v != 1 && v != -1) return fail(c, J1J2C_EINVAL, "spins must be +1 or -1");
                const int ci = compact_of_site(g, s);
                buf[(size_t)r * c->lat_stride + ci] = occ[ci] ? (uint8_t)(v + 1) : (uint8_t)1;
            }
        CK(c, cudaMemcpy(dst, buf.data(), buf.size(), cudaMemcpyHostToDevice));
    } else {
        InitArgs a{};
        a.g = g;
        a.spins = dst;
        a.lat_stride = c->lat_stride;
        a.occ = c->d_occ + (size_t)conf * c->lat_stride;
        a.nrep = c->nrep;
        a.start = start;
        a.axis = axis;
        a.seed = c->P.seed;
        a.key1 = c->P.conf_base + (uint32_t)conf;
        CK(c, launch_init(a, c->st));
    }
    // Initialize_pt_state: identity maps, swap counters zeroed (J:1222-1233)
    CK(c, cudaMemsetAsync(c->d_att + (size_t)conf * c->nrep, 0, sizeof(long long) * c->nrep, c->st));
    CK(c, cudaMemsetAsync(c->d_acc + (size_t)conf * c->nrep, 0, sizeof(long long) * c->nrep, c->st));
    std::vector<int> ident((size_t)c->nrep);
    for (int r = 0; r < c->nrep; ++r) ident[r] = r;
    CK(c, cudaMemcpyAsync(c->d_rat + (size_t)conf * c->nrep, ident.data(), sizeof(int) * c->nrep,
                          cudaMemcpyHostToDevice, c->st));
    CK(c, cudaMemcpyAsync(c->d_tor + (size_t)conf * c->nrep, ident.data(), sizeof(int) * c->nrep,
                          cudaMemcpyHostToDevice, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    c->have_spins[conf] = 1;
    return J1J2C_OK;
}

int j1j2c_reset_measurements(void* ctx, int32_t conf)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (conf >= c->nconf) return fail(c, J1J2C_EINVAL, "conf out of range");
    const int c0 = conf < 0 ? 0 : conf, c1 = conf < 0 ? c->nconf : conf + 1;
    const size_t n = (size_t)(c1 - c0) * c->nrep, off = (size_t)c0 * c->nrep;
    std::vector<double> sums(n * 22, 0.0);
    for (size_t k = 0; k < n; ++k) sums[k * 22 + 20] = std::numeric_limits<double>::infinity();
    CK(c, cudaMemcpy(c->d_sums + off * 22, sums.data(), sums.size() * 8, cudaMemcpyHostToDevice));
    CK(c, cudaMemset(c->d_nmeas + off, 0, n * sizeof(long long)));
    CK(c, cudaMemset(c->d_vis + off, 0, n));
    return J1J2C_OK;
}

int j1j2c_run(void* ctx, int32_t ncycles, int32_t measure, int32_t restart_swap_phase)
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
    int rct = autotune(c);
    if (rct != J1J2C_OK) return rct;
    const bool direct = (c->P.flags & J1J2C_FLAG_NO_GRAPH) != 0;
    if (!direct && !c->graph[m]) {
        int rc = build_graph(c, m);
        if (rc != J1J2C_OK) return rc;
    }
    for (int k = 0; k < ncycles; ++k) {
        if (direct)
            CK(c, enqueue_cycle(c, m, c->st));
        else
            CK(c, cudaGraphLaunch(c->graph[m], c->st));
        if (c->profile) {  // the events bracket the sweep kernel (graph event-record nodes)
            CK(c, cudaEventSynchronize(c->ev1));
            float ms = 0.0f;
            CK(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            c->prof_ms += ms;
            c->prof_launches += 1;
            c->prof_attempts += c->occ_total * c->P.ptswapever;
        }
    }
    CK(c, cudaStreamSynchronize(c->st));
    CK(c, cudaGetLastError());
    return J1J2C_OK;
}

int j1j2c_metro_sweep_fp64(void* ctx, int32_t conf, int32_t rep, double beta,
                           uint32_t sweep_index, int32_t nsweeps, double* mag, double* en,
                           double* strx, double* stry)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf) || rep < 0 || rep >= c->nrep)
        return fail(c, J1J2C_EINVAL, "conf or replica out of range");
    if (!c->have_dis[conf] || !c->have_spins[conf])
        return fail(c, J1J2C_ESTATE, "conf lacks disorder or spins");
    if (nsweeps < 0 || !std::isfinite(beta) || beta < 0.0)
        return fail(c, J1J2C_EINVAL, "bad nsweeps or beta");
    SweepVariant v;
    size_t smem;
    int nt;
    int rc = choose_variant(c, true, v, smem, nt);
    if (rc != J1J2C_OK) return rc;
    SweepArgs a = base_args(c);
    a.lat0 = conf * c->nrep + rep;
    a.nsweeps = nsweeps;
    a.use_override = 1;
    a.beta_override = beta;
    a.sweep_override = sweep_index;
    CK(c, launch_sweep(a, v, 1, nt, smem, c->st));
    LatObs o;
    CK(c, cudaMemcpyAsync(&o, c->d_obs + a.lat0, sizeof o, cudaMemcpyDeviceToHost, c->st));
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
    SweepVariant v{};
    v.fp64 = true;
    v.quad = false;
    v.stage_p = false;
    v.masks = c->masks;
    v.mode = kModeAudit;
    const size_t smem = sweep_smem_bytes(c->g, v);
    CK(c, prepare_sweep_variant(v, smem));
    int nt = ((c->g.Nc + 31) / 32) * 32;
    if (nt > 512) nt = 512;
    if (nt < 64) nt = 64;
    CK(c, cudaMemsetAsync(c->d_audit, 0, 2 * sizeof(unsigned long long), c->st));
    SweepArgs a = base_args(c);
    a.nsweeps = nsweeps;
    CK(c, launch_sweep(a, v, c->nlat, nt, smem, c->st));
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
    const size_t off = conf < 0 ? 0 : (size_t)conf * c->nrep;
    const int nr = (conf < 0 ? c->nconf : 1) * c->nrep;
    std::vector<double> sums((size_t)nr * 22);
    std::vector<long long> nm((size_t)nr);
    CK(c, cudaMemcpyAsync(sums.data(), c->d_sums + off * 22, sums.size() * 8,
                          cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaMemcpyAsync(nm.data(), c->d_nmeas + off, nm.size() * 8, cudaMemcpyDeviceToHost,
                          c->st));
    CK(c, cudaStreamSynchronize(c->st));
    for (int r = 0; r < nr; ++r) {
        std::memcpy(&out[r], &sums[(size_t)r * 22], 22 * sizeof(double));
        out[r].nmeasure = nm[r];
    }
    return J1J2C_OK;
}

int j1j2c_get_pt_stats(void* ctx, int32_t conf, int64_t* attempts, int64_t* accepts,
                       int32_t* visited_both)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!valid_conf(c, conf)) return fail(c, J1J2C_EINVAL, "conf out of range");
    const size_t off = (size_t)conf * c->nrep;
    std::vector<long long> at((size_t)c->nrep), ac((size_t)c->nrep);
    std::vector<uint8_t> vis((size_t)c->nrep);
    CK(c, cudaMemcpyAsync(at.data(), c->d_att + off, at.size() * 8, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaMemcpyAsync(ac.data(), c->d_acc + off, ac.size() * 8, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaMemcpyAsync(vis.data(), c->d_vis + off, vis.size(), cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    for (int k = 0; k + 1 < c->nrep; ++k) {
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
    const size_t off = (size_t)conf * c->nrep, nb = sizeof(int) * c->nrep;
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
    if (!valid_conf(c, conf) || rep < 0 || rep >= c->nrep || !out)
        return fail(c, J1J2C_EINVAL, "bad conf, replica or output");
    const Geo& g = c->g;
    std::vector<uint8_t> buf((size_t)g.N);
    CK(c, cudaMemcpyAsync(buf.data(), c->d_spins + ((size_t)conf * c->nrep + rep) * c->lat_stride,
                          g.N, cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
    for (int s = 0; s < g.N; ++s) out[s] = (int8_t)((int)buf[compact_of_site(g, s)] - 1);
    return J1J2C_OK;
}

int j1j2c_get_observables(void* ctx, int32_t conf, double* out)
{
    if (!ctx) return J1J2C_EINVAL;
    Ctx* c = static_cast<Ctx*>(ctx);
    if (conf >= c->nconf || !out) return fail(c, J1J2C_EINVAL, "bad conf or null output");
    const size_t off = conf < 0 ? 0 : (size_t)conf * c->nrep;
    const size_t nr = (size_t)(conf < 0 ? c->nconf : 1) * c->nrep;
    CK(c, cudaMemcpyAsync(out, c->d_last + off * 5, sizeof(double) * 5 * nr,
                          cudaMemcpyDeviceToHost, c->st));
    CK(c, cudaStreamSynchronize(c->st));
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
    if (block_threads) *block_threads = c->nthreads;
    if (sites_per_thread) *sites_per_thread = c->var.quad ? 4 : 1;
    if (smem_bytes) *smem_bytes = (int32_t)c->smem;
    return J1J2C_OK;
}

}  // extern "C"
