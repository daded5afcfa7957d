// Diagonal densities of an operator over a subsystem (the reference's DiagDensityOp,
// source/network_functions/DiagDensityOp.cu:12-50): for every configuration s of the
// ensemble, |E_loc(s)|^2 times its weight is added to the bin of the configuration of
// the first N_A spins (the low N_A bits, include/Spins.h:255-257).  A block histograms its
// samples in shared memory (FP64 atomics) and adds the bins to the output once.
#include "host.h"

namespace rbmg {

namespace {

constexpr int kMaxSharedBins = 4096;   // 32 KB of doubles

__global__ void diag_density_kernel(int count, int enumerate, uint64_t enum_base, const uint64_t* spins, int nw,
                                    const double* w, const double2* eloc, int na, double* out) {
    __shared__ double hist[kMaxSharedBins];
    const int bins = 1 << na;
    const bool shared = bins <= kMaxSharedBins;
    if (shared)
        for (int i = threadIdx.x; i < bins; i += blockDim.x) hist[i] = 0.0;
    __syncthreads();
    const uint64_t mask = na >= 64 ? ~0ull : ((1ull << na) - 1ull);
    for (long s = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x; s < count;
         s += static_cast<long>(gridDim.x) * blockDim.x) {
        const uint64_t word = enumerate ? enum_base + static_cast<uint64_t>(s) : spins[s * nw];
        const int bin = static_cast<int>(word & mask);
        const double2 e = eloc[s];
        const double v = (w ? w[s] : 1.0) * (e.x * e.x + e.y * e.y);
        if (shared) atomicAdd(&hist[bin], v);
        else atomicAdd(&out[bin], v);
    }
    if (!shared) return;
    __syncthreads();
    for (int i = threadIdx.x; i < bins; i += blockDim.x)
        if (hist[i] != 0.0) atomicAdd(&out[i], hist[i]);
}

__global__ void sub_kernel(int count, const double2* a, const double2* b, double2* out) {
    for (long s = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x; s < count;
         s += static_cast<long>(gridDim.x) * blockDim.x)
        out[s] = make_double2(a[s].x - b[s].x, a[s].y - b[s].y);
}

}  // namespace

cudaError_t launch_sub(int count, const double2* a, const double2* b, double2* out, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    sub_kernel<<<std::min((count + 255) / 256, 4096), 256, 0, st>>>(count, a, b, out);
    return cudaGetLastError();
}

cudaError_t launch_diag_density(int count, int enumerate, uint64_t enum_base, const uint64_t* spins, int nw,
                                const double* w, const double2* eloc, int na, double* out, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const int blocks = std::min((count + 255) / 256, 1024);
    diag_density_kernel<<<blocks, 256, 0, st>>>(count, enumerate, enum_base, spins, nw, w, eloc, na, out);
    return cudaGetLastError();
}

}  // namespace rbmg
