// Disorder generation on the GPU: make_corr_rand_3d (CR:191-386) with the three 3-D transforms,
// the filter and the crop on the device (cuFFT, double complex), the white noise drawn on the
// host (one sequential gkiss05 stream in the reference's order, CR:280-287) and the uniform map
// applied on the host.  Same steps as the host form j1j2c_corr_rand_3d; the two agree to the
// rounding of the transforms (~1e-15).
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/j1j2c.h"
#include "engine.h"

namespace j1j2 {
void gauss_fill(int32_t seed, size_t n, double* out);
double uniform_map(double v, double max_value);
}  // namespace j1j2

namespace {

int pow2_at_least(int n)
{
    int p = 1;
    while (p < n) p *= 2;
    return p;
}

// C(dx,dy,dz) = exp(-r/xi) with the periodic distance on the padded cube (CR:261-268, 362-384)
__global__ void filter_kernel(cufftDoubleComplex* c, int f1, int f2, int f3, double xi)
{
    const size_t nt = (size_t)f1 * f2 * f3;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int i = (int)(t % (size_t)f1), j = (int)((t / (size_t)f1) % (size_t)f2);
    const int k = (int)(t / ((size_t)f1 * f2));
    const int dx = i < f1 - i ? i : f1 - i, dy = j < f2 - j ? j : f2 - j, dz = k < f3 - k ? k : f3 - k;
    const double r = sqrt((double)(dx * dx + dy * dy + dz * dz));
    const double v = xi <= 0.0 ? (r == 0.0 ? 1.0 : 0.0) : exp(-r / xi);
    c[t] = make_cuDoubleComplex(v, 0.0);
}

__global__ void noise_kernel(const double* x, cufftDoubleComplex* X, size_t nt)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nt) X[t] = make_cuDoubleComplex(x[t], 0.0);
}

// X_k <- X_k * sqrt(|Re C_k|) (CR:303-310)
__global__ void shape_kernel(cufftDoubleComplex* X, const cufftDoubleComplex* C, size_t nt)
{
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const double w = sqrt(fabs(C[t].x));
    X[t] = make_cuDoubleComplex(X[t].x * w, X[t].y * w);
}

__global__ void crop_kernel(const cufftDoubleComplex* X, double* out, int n1, int n2, int n3,
                            int f1, int f2, double scale)
{
    const size_t n = (size_t)n1 * n2 * n3;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = (int)(t % (size_t)n1), j = (int)((t / (size_t)n1) % (size_t)n2);
    const int k = (int)(t / ((size_t)n1 * n2));
    out[t] = X[((size_t)k * f2 + j) * f1 + i].x * scale;
}

unsigned blocks(size_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

extern "C" int j1j2c_corr_rand_3d_gpu(int32_t n1, int32_t n2, int32_t n3, double xi,
                                      int32_t seed, int32_t do_uniform, double max_value,
                                      double* out)
{
    if (n1 < 1 || n2 < 1 || n3 < 1 || !out) {
        j1j2::set_global_error("j1j2c_corr_rand_3d_gpu: bad extents or null output");
        return J1J2C_EINVAL;
    }
    const int f1 = pow2_at_least(n1), f2 = pow2_at_least(n2), f3 = pow2_at_least(n3);
    const size_t nt = (size_t)f1 * f2 * f3, n = (size_t)n1 * n2 * n3;
    if (nt > ((size_t)1 << 27)) {
        j1j2::set_global_error("j1j2c_corr_rand_3d_gpu: padded cube too large");
        return J1J2C_EINVAL;
    }
    std::vector<double> noise(nt);
    j1j2::gauss_fill(seed, nt, noise.data());
    cufftDoubleComplex *C = nullptr, *X = nullptr;
    double *xd = nullptr, *od = nullptr;
    cufftHandle plan = 0;
    bool have_plan = false;
    int rc = J1J2C_OK;
    std::string what;
    auto ck = [&](cudaError_t e, const char* w) {
        if (rc == J1J2C_OK && e != cudaSuccess) {
            rc = e == cudaErrorMemoryAllocation ? J1J2C_ENOMEM : J1J2C_ECUDA;
            what = std::string(w) + ": " + cudaGetErrorString(e);
        }
        return rc == J1J2C_OK;
    };
    auto fk = [&](cufftResult r, const char* w) {
        if (rc == J1J2C_OK && r != CUFFT_SUCCESS) {
            rc = J1J2C_ECUDA;
            what = std::string(w) + ": cuFFT error " + std::to_string((int)r);
        }
        return rc == J1J2C_OK;
    };
    if (ck(cudaMalloc(&C, nt * sizeof(cufftDoubleComplex)), "cudaMalloc") &&
        ck(cudaMalloc(&X, nt * sizeof(cufftDoubleComplex)), "cudaMalloc") &&
        ck(cudaMalloc(&xd, nt * sizeof(double)), "cudaMalloc") &&
        ck(cudaMalloc(&od, n * sizeof(double)), "cudaMalloc") &&
        ck(cudaMemcpy(xd, noise.data(), nt * sizeof(double), cudaMemcpyHostToDevice), "noise") &&
        fk(cufftPlan3d(&plan, f3, f2, f1, CUFFT_Z2Z), "cufftPlan3d")) {
        have_plan = true;
        filter_kernel<<<blocks(nt), 256>>>(C, f1, f2, f3, xi);
        noise_kernel<<<blocks(nt), 256>>>(xd, X, nt);
        if (ck(cudaGetLastError(), "filter / noise") &&
            fk(cufftExecZ2Z(plan, C, C, CUFFT_FORWARD), "forward transform of the filter") &&
            fk(cufftExecZ2Z(plan, X, X, CUFFT_FORWARD), "forward transform of the noise")) {
            shape_kernel<<<blocks(nt), 256>>>(X, C, nt);
            if (ck(cudaGetLastError(), "filter product") &&
                fk(cufftExecZ2Z(plan, X, X, CUFFT_INVERSE), "inverse transform")) {
                crop_kernel<<<blocks(n), 256>>>(X, od, n1, n2, n3, f1, f2, 1.0 / (double)nt);
                if (ck(cudaGetLastError(), "crop"))
                    ck(cudaMemcpy(out, od, n * sizeof(double), cudaMemcpyDeviceToHost), "result");
            }
        }
    }
    if (have_plan) cufftDestroy(plan);
    cudaFree(C);
    cudaFree(X);
    cudaFree(xd);
    cudaFree(od);
    if (rc != J1J2C_OK) {
        j1j2::set_global_error(("j1j2c_corr_rand_3d_gpu: " + what).c_str());
        return rc;
    }
    if (do_uniform)
        for (size_t t = 0; t < n; ++t) out[t] = j1j2::uniform_map(out[t], max_value);
    return J1J2C_OK;
}
