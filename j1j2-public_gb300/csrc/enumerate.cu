// Exact Boltzmann averages of a small lattice (N <= 32 sites, e.g. 4 x 4 x 2) by enumerating
// all 2^N spin states on the GPU: the oracle for the sampled averages of the Metropolis, PT and
// Wolff updates.  No reference counterpart (the reference only samples).
//
// State bit i is the spin of site i (reference site order, 1 = up).  Each thread fixes the high
// N - LB bits and walks the low LB bits in Gray-code order, so consecutive states differ by one
// spin: the energy changes by 2 s_i field_i with the FP64 local field of Compute_local_field
// (J:2498-2541) and m, the stripe sums and the nematic sum change by closed-form increments.
// For every beta the kernel accumulates, with weights w = exp(-beta (E - E0)) (E0 a lower bound
// of E, so w <= 1), the sums of w, w E, w E^2, w |m|, w m^2, w m^4, w |sx|, w sx^2, w |sy|, w sy^2,
// w nbar, w nbar^2 (per-site observables as in Measurement, J:2807-2842, and J:1028-1048).
#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/j1j2c.h"
#include "engine.h"

namespace j1j2 {

namespace {

__device__ __forceinline__ int spin_of(uint32_t state, int i) { return ((state >> i) & 1u) ? 1 : -1; }

__device__ double local_field(const EnumArgs& a, uint32_t state, int i)
{
    Nbr64 n;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        const int j = a.nbr[i][k];
        n.s[k] = a.occ[j] ? spin_of(state, j) : 0;
    }
    n.p1 = a.p[a.nbr[i][0]];
    n.p2 = a.p[a.nbr[i][1]];
    n.p3 = a.p[a.nbr[i][2]];
    n.p4 = a.p[a.nbr[i][3]];
    n.jv_own = a.jv[i];
    n.jv_m2 = a.jv[a.nbr[i][1]];
    n.jh_own = a.jh[i];
    n.jh_m4 = a.jh[a.nbr[i][3]];
    return field_fp64(n, a.p[i], a.J1h, a.J1v, a.J2, a.J3, nullptr);
}

// nematic term of site i: s_+x + s_-x - s_+y - s_-y over occupied neighbours
__device__ __forceinline__ int nem_of(const EnumArgs& a, uint32_t state, int i)
{
    int v = 0;
    const int jx1 = a.nbr[i][2], jx2 = a.nbr[i][3], jy1 = a.nbr[i][0], jy2 = a.nbr[i][1];
    v += a.occ[jx1] ? spin_of(state, jx1) : 0;
    v += a.occ[jx2] ? spin_of(state, jx2) : 0;
    v -= a.occ[jy1] ? spin_of(state, jy1) : 0;
    v -= a.occ[jy2] ? spin_of(state, jy2) : 0;
    return v;
}

__global__ void __launch_bounds__(128) enumerate_kernel(EnumArgs a, double* partial)
{
    const uint32_t hi = (uint32_t)(blockIdx.x * blockDim.x + threadIdx.x);
    const bool active = hi < (1u << (a.N - a.LB));
    double acc[kEnumBeta][kEnumSums];
#pragma unroll
    for (int b = 0; b < kEnumBeta; ++b)
#pragma unroll
        for (int q = 0; q < kEnumSums; ++q) acc[b][q] = 0.0;
    if (active) {
        uint32_t state = hi << a.LB;
        double E = 0.0;
        int M = 0, SX = 0, SY = 0, NB = 0;
        for (int i = 0; i < a.N; ++i) {
            if (!a.occ[i]) continue;
            const int s = spin_of(state, i);
            E = __dadd_rn(E, -((double)s * local_field(a, state, i)));
            M += s;
            SX += a.px[i] ? -s : s;
            SY += a.py[i] ? -s : s;
            NB += s * nem_of(a, state, i);
        }
        E = __dmul_rn(E, 0.5);
        const uint32_t nlow = 1u << a.LB;
        for (uint32_t k = 0;; ++k) {
            const double e = E / a.nocc, m = (double)M / a.nocc, sx = (double)SX / a.nocc,
                         sy = (double)SY / a.nocc, nb = (double)NB / a.nocc;
            const double m2 = m * m, e2 = e * e;
#pragma unroll
            for (int b = 0; b < kEnumBeta; ++b) {
                if (b >= a.nbeta) break;
                const double w = own_exp(-a.beta[b] * (E - a.E0));
                acc[b][0] += w;
                acc[b][1] += w * e;
                acc[b][2] += w * e2;
                acc[b][3] += w * fabs(m);
                acc[b][4] += w * m2;
                acc[b][5] += w * m2 * m2;
                acc[b][6] += w * fabs(sx);
                acc[b][7] += w * sx * sx;
                acc[b][8] += w * fabs(sy);
                acc[b][9] += w * sy * sy;
                acc[b][10] += w * nb;
                acc[b][11] += w * nb * nb;
            }
            if (k + 1 == nlow) break;
            const int i = __ffs((int)(k + 1)) - 1;  // Gray code: bit flipped at step k+1
            if (a.occ[i]) {
                const int s = spin_of(state, i);
                E = __dadd_rn(E, __dmul_rn(2.0 * s, local_field(a, state, i)));
                M -= 2 * s;
                SX -= 2 * (a.px[i] ? -s : s);
                SY -= 2 * (a.py[i] ? -s : s);
                NB -= 4 * s * nem_of(a, state, i);
            }
            state ^= 1u << i;
        }
    }
    // block reduction (fixed order) into this block's partial sums
    __shared__ double red[128];
#pragma unroll
    for (int b = 0; b < kEnumBeta; ++b)
#pragma unroll
        for (int q = 0; q < kEnumSums; ++q) {
            if (b >= a.nbeta) continue;  // uniform across the block
            red[threadIdx.x] = acc[b][q];
            __syncthreads();
            for (int o = 64; o > 0; o >>= 1) {
                if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
                __syncthreads();
            }
            if (threadIdx.x == 0) partial[((size_t)blockIdx.x * kEnumBeta + b) * kEnumSums + q] = red[0];
            __syncthreads();
        }
}

}  // namespace

int enum_blocks(const EnumArgs& a)
{
    const uint32_t threads = 1u << (a.N - a.LB);
    return (int)((threads + 127) / 128);
}

cudaError_t launch_enumerate(const EnumArgs& a, double* partial, cudaStream_t st)
{
    enumerate_kernel<<<enum_blocks(a), 128, 0, st>>>(a, partial);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------------
// Allocation-free variant (j1j2c_enumerate_exact_noalloc).  Some callers cannot create device
// allocations at the moment they need the exact averages: a host program whose memory manager has
// already reserved the whole GPU for its own pool (a new cudaMalloc fails or fragments that
// pool), or a latency-bound loop that must not pay for an allocation and its implicit
// synchronisation.  This variant keeps the per-block partial sums and their total in one fixed
// device array instead of a buffer allocated per call.
//
// Limit: 512 CTAs (the 2^16 threads of a 32-site lattice, 128 per CTA) x 4 inverse temperatures
// x 12 sums of partials, plus 48 totals: 24624 doubles (about 192 KiB), held by every GPU that
// loads the library until the process exits.  All calls share the array and overwrite it (every
// entry a call reads was written earlier in that call, so nothing needs clearing); calls that
// overlap on the GPU, from two host threads or two processes' streams, race on it.
// ------------------------------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxBlocks = 512;
constexpr int kNoAllocPartials = kNoAllocMaxBlocks * kEnumBeta * kEnumSums;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_enum_scratch[kNoAllocPartials + kEnumBeta * kEnumSums];

// totals[b * 12 + q] = sum over blocks of partial[(blk * 4 + b) * 12 + q], in block order
__global__ void enum_total_kernel(const double* partial, int nblocks, int nbeta, double* totals)
{
    const int t = (int)threadIdx.x;
    if (t < nbeta * kEnumSums) {
        const int b = t / kEnumSums, q = t - b * kEnumSums;
        double s = 0.0;
        for (int blk = 0; blk < nblocks; ++blk)
            s += partial[((size_t)blk * kEnumBeta + b) * kEnumSums + q];
        totals[t] = s;
    }
}

std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_enum_scratch on the current device, looked up once per device.  In host
// code the symbol is only a host-side stand-in, so the kernel must receive this address.  The
// address is kept for the life of the process: a cudaDeviceReset between calls (which unloads
// the module and with it the array) is not supported.
cudaError_t scratch_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_enum_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

}  // namespace j1j2

extern "C" int j1j2c_enumerate_exact_noalloc(int32_t L, int32_t H, double J1h, double J1v,
                                             double J2, double J3, const double* p,
                                             const int8_t* occu, const int8_t* jh,
                                             const int8_t* jv, int32_t nbeta, const double* beta,
                                             double* out)
{
    using namespace j1j2;
    set_global_error("");  // j1j2c_last_error(NULL) reports this call's outcome only
    const int N = L * L * H;
    if (L < 2 || H < 2 || (L & 1) || (H & 1) || N > 32 || !p || !beta || !out || nbeta < 1 ||
        nbeta > kEnumBeta) {
        set_global_error("allocation-free enumeration: needs even L, H with L*L*H <= 32 sites "
                         "and 1..4 inverse temperatures");
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
        if (!std::isfinite(p[i])) {
            set_global_error("allocation-free enumeration: p must be finite");
            return J1J2C_EINVAL;
        }
        const int x = i % L, y = (i / L) % L, z = i / (L * L);
        const int dx[10] = {0, 0, 1, -1, 1, -1, 1, -1, 0, 0};
        const int dy[10] = {1, -1, 0, 0, 1, 1, -1, -1, 0, 0};
        const int dz[10] = {0, 0, 0, 0, 0, 0, 0, 0, 1, -1};
        for (int k = 0; k < 10; ++k)
            a.nbr[i][k] = (int8_t)(((x + dx[k] + L) % L) + L * ((y + dy[k] + L) % L) +
                                   L * L * ((z + dz[k] + H) % H));
        a.p[i] = p[i];
        a.occ[i] = occu ? (occu[i] != 0) : 1;
        a.jh[i] = jh ? (jh[i] != 0) : 1;
        a.jv[i] = jv ? (jv[i] != 0) : 1;
        a.px[i] = (uint8_t)(x & 1);
        a.py[i] = (uint8_t)(y & 1);
        nocc += a.occ[i];
        pmax = std::fmax(pmax, std::fabs(p[i]));
    }
    if (nocc == 0) {
        set_global_error("allocation-free enumeration: no occupied site");
        return J1J2C_EINVAL;
    }
    a.nocc = (double)nocc;
    a.E0 = -0.5 * N *
               (2 * std::fabs(J1h) + 2 * std::fabs(J1v) + 4 * std::fabs(J2) +
                2 * std::fabs(J3) + 8 * pmax) -
           1.0;
    for (int b = 0; b < nbeta; ++b) {
        if (!std::isfinite(beta[b]) || beta[b] < 0.0) {
            set_global_error("allocation-free enumeration: beta must be finite and >= 0");
            return J1J2C_EINVAL;
        }
        a.beta[b] = beta[b];
    }
    const int nb = enum_blocks(a);
    if (nb > kNoAllocMaxBlocks) {
        set_global_error("allocation-free enumeration: more than 512 CTAs of partial sums");
        return J1J2C_EINVAL;
    }
    double* scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e == cudaSuccess) e = launch_enumerate(a, scratch, 0);
    if (e == cudaSuccess) {
        enum_total_kernel<<<1, kEnumBeta * kEnumSums>>>(scratch, nb, nbeta,
                                                        scratch + kNoAllocPartials);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(out, scratch + kNoAllocPartials, sizeof(double) * kEnumSums * nbeta,
                       cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        thread_local char msg[192];
        std::snprintf(msg, sizeof msg, "allocation-free enumeration: %s", cudaGetErrorString(e));
        set_global_error(msg);
        return J1J2C_ECUDA;
    }
    for (int b = 0; b < nbeta; ++b) {  // totals -> ln Z and averages, in place
        double* o = out + (size_t)b * kEnumSums;
        const double z = o[0];
        for (int q = 1; q < kEnumSums; ++q) o[q] = o[q] / z;
        o[0] = std::log(z) - beta[b] * a.E0;
    }
    return 0;
}
