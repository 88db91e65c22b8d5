// Helpers shared by the generic sweep kernels (kernels.cu) and the shape-specialised sweep
// kernels (sweep_fixed.cu): per-thread reduction state, block reduction, word shifts for the
// +-x neighbours, fixed-point energy terms, and lattice staging between HBM and shared memory.
#pragma once
#include "engine.h"

namespace j1j2 {

// random field of configuration conf (compact layout)
template <class Real>
__device__ __forceinline__ const Real* field_base(const SweepArgs& a, int conf)
{
    if constexpr (sizeof(Real) == 8)
        return a.pd + (long long)conf * a.p_stride;
    else
        return a.pf + (long long)conf * a.p_stride;
}

struct Acc {
    long long e;  // fixed-point energy, sum of llrint(-s*field * 2^32)
    int M, SX, SY, NB;
};

__device__ __forceinline__ int wrap_p(int v, int n) { return v + 1 == n ? 0 : v + 1; }
__device__ __forceinline__ int wrap_m(int v, int n) { return v == 0 ? n - 1 : v - 1; }

// fixed-point energy contribution of one site: llrint(e * 2^32) for |e| < 2^30, rounded from
// e's bits in integer arithmetic (no FP64 operation): e 2^32 = m 2^(ex - 1043) with m the 53-bit
// significand, rounded to nearest, ties to even, when the shift drops bits
__device__ __forceinline__ long long efix(double e)
{
    const long long bits = __double_as_longlong(e);
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex == 0) return 0;  // zero, or subnormal (|e 2^32| < 2^-990)
    const long long m = (bits & 0xFFFFFFFFFFFFFLL) | 0x10000000000000LL;
    const int sh = 1043 - ex;
    long long v;
    if (sh <= 0) {
        v = m << (-sh);  // integral
    } else if (sh > 53) {
        v = 0;           // below 1/2
    } else {
        const long long q = m >> sh, r = m & ((1LL << sh) - 1), half = 1LL << (sh - 1);
        v = q + ((r > half || (r == half && (q & 1))) ? 1 : 0);
    }
    return bits < 0 ? -v : v;
}
// same value for an FP32 energy term: e * 2^32 is exact in FP32, so no FP64 operation is needed
__device__ __forceinline__ long long efix32(float e)
{
    return __float2ll_rn(__fmul_rn(e, 4294967296.0f));
}

// efix32 without the 64-bit conversion (which runs on the FP64 pipe): with x = e * 2^16,
// t = trunc(x) and r = x - t (exact), llrint(e * 2^32) = t * 2^16 + rint(r * 2^16) because
// t * 2^16 is an even integer, so rounding (ties to even included) only acts on r * 2^16.
// |t| < 2^23 for |e| < 2^7, so both parts fit 32-bit conversions.
__device__ __forceinline__ long long efix32_split(float e)
{
    const float x = __fmul_rn(e, 65536.0f);
    const float t = truncf(x);
    const int hi = __float2int_rz(t);
    const int lo = __float2int_rn(__fmul_rn(__fsub_rn(x, t), 65536.0f));
    return ((long long)hi << 16) + (long long)lo;
}

// Neighbour words along x for a run of four compact X of one colour.  A is the word with the
// same X range in the neighbouring colour, B the next (px = 1) or previous (px = 0) word.
__device__ __forceinline__ void x_pair(int px, uint32_t A, uint32_t B, uint32_t& plus,
                                       uint32_t& minus)
{
    if (px) {  // site X: +x neighbour at compact X+1, -x at X
        minus = A;
        plus = __byte_perm(A, B, 0x4321);
    } else {  // +x at X, -x at X-1
        plus = A;
        minus = __byte_perm(B, A, 0x6543);
    }
}

// Packed FP32 pairs (Blackwell add/sub/mul/fma .f32x2: two IEEE round-to-nearest operations per
// instruction, element by element)
using f2 = unsigned long long;

__device__ __forceinline__ f2 f2_pack(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ f2 f2_splat(float v) { return f2_pack(v, v); }
__device__ __forceinline__ float f2_get(f2 v, int e)
{
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return e ? hi : lo;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c)
{
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// bytes k and k+1 of w as 2^23 + byte (exact floats; subtract 2^23 + offset afterwards)
__device__ __forceinline__ f2 byte_pair(uint32_t w, int k)
{
    return f2_pack(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + (uint32_t)k)),
                   __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7541u + (uint32_t)k)));
}

// Raise a kernel's dynamic shared memory limit to the most the device allows next to its static
// shared memory (one instantiation may serve several shapes and sizes in one context).
template <class Kernel>
inline cudaError_t raise_smem_limit(Kernel kern)
{
    int dev = 0, optin = 0;
    cudaFuncAttributes fa{};
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kern);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa.sharedSizeBytes);
    return e;
}

// byte k of w minus off, as an exact float (one PRMT into a 2^23 exponent field, one FADD)
__device__ __forceinline__ float byte_off(uint32_t w, int k, float off)
{
    return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + (uint32_t)k)),
                     8388608.0f + off);
}

__device__ __forceinline__ void warp_reduce(Acc& v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.e += __shfl_down_sync(0xFFFFFFFFu, v.e, o);
        v.M += __shfl_down_sync(0xFFFFFFFFu, v.M, o);
        v.SX += __shfl_down_sync(0xFFFFFFFFu, v.SX, o);
        v.SY += __shfl_down_sync(0xFFFFFFFFu, v.SY, o);
        v.NB += __shfl_down_sync(0xFFFFFFFFu, v.NB, o);
    }
}

// block-wide sum; the result is valid in thread 0
__device__ __forceinline__ Acc block_reduce(Acc v)
{
    __shared__ Acc red[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    warp_reduce(v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? red[lane] : Acc{0, 0, 0, 0, 0};
        warp_reduce(v);
    }
    return v;
}

__device__ __forceinline__ void store_obs(LatObs* out, const Acc& t)
{
    LatObs o;
    o.eacc = t.e;
    o.M = t.M;
    o.SX = t.SX;
    o.SY = t.SY;
    o.NB = t.NB;
    o.pad[0] = o.pad[1] = 0;
    *out = o;
}

// 16-byte vector copy of nbytes (a multiple of 16) by the whole block
__device__ __forceinline__ void block_copy16(void* dst, const void* src, int nbytes)
{
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (int k = (int)threadIdx.x; k < nbytes / 16; k += (int)blockDim.x) d[k] = s[k];
}

__device__ __forceinline__ void block_copy16_ldg(void* dst, const void* src, int nbytes)
{
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (int k = (int)threadIdx.x; k < nbytes / 16; k += (int)blockDim.x) d[k] = __ldg(s + k);
}

// ---- bulk copies through the tensor memory accelerator, completed on an mbarrier -----------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// one arrival that also announces the bytes the pending copies will deliver
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase with the given parity to complete; gives up after a bounded number of tries
// (then flags err and returns false: the data is not there, nothing hangs)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err)
{
    for (int it = 0; it < (1 << 20); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    if (err) atomicExch(err, 1);
    return false;
}

// global -> shared, bytes a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// shared -> global, bytes a multiple of 16, both addresses 16-byte aligned
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                 "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit()
{
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// the bulk stores issued so far have read their shared memory
__device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// the bulk stores issued so far are complete
__device__ __forceinline__ void bulk_wait_all()
{
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// order this thread's shared-memory accesses before later bulk copies (the async proxy)
__device__ __forceinline__ void fence_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Programmatic dependent launch.  A kernel launched with the programmatic-serialisation attribute
// may be scheduled while the previous kernel of its stream still runs; pdl_wait() returns once
// that kernel has completed and its memory operations are visible (in a kernel launched without
// the attribute it returns at once).  Every kernel launched through launch_k with pdl set calls
// pdl_wait() before its first global-memory access.  pdl_release() lets the next such kernel be
// scheduled as soon as every CTA of this one has started.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ void pdl_release()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <class... P, class... A>
cudaError_t launch_k(bool pdl, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     void (*kernel)(P...), A&&... args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1u : 0u;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<A&&>(args)...);
}

}  // namespace j1j2
