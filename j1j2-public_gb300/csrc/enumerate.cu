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

}  // namespace j1j2
