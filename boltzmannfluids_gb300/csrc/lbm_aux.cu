// lbm_aux.cu -- thermal lattice kernels (D2Q5 / D3Q7) and the second pass of
// the FP64 conservation reduction.
#include "lbm_kernels.cuh"

namespace bf {

// the FP64 stepper's thermal lattice is double (src64 / th64 set), every
// other storage's FP32
template <int QT>
cudaError_t launch_stream_thermal(const ThermalStreamParams& p, cudaStream_t st) {
    int block;
    dim3 grid = cell_grid(p.nx, p.ny, p.nz, block);
    if (p.src64) stream_thermal_kernel<QT, double><<<grid, block, 0, st>>>(p);
    else stream_thermal_kernel<QT, float><<<grid, block, 0, st>>>(p);
    return cudaGetLastError();
}
template <int QT>
cudaError_t launch_init_thermal(const InitParams& p, cudaStream_t st) {
    const unsigned blocks = (unsigned)((p.n_cells + 255u) / 256u);
    if (p.th64) init_thermal_kernel<QT, double><<<blocks, 256, 0, st>>>(p);
    else init_thermal_kernel<QT, float><<<blocks, 256, 0, st>>>(p);
    return cudaGetLastError();
}
template cudaError_t launch_stream_thermal<5>(const ThermalStreamParams&, cudaStream_t);
template cudaError_t launch_stream_thermal<7>(const ThermalStreamParams&, cudaStream_t);
template cudaError_t launch_init_thermal<5>(const InitParams&, cudaStream_t);
template cudaError_t launch_init_thermal<7>(const InitParams&, cudaStream_t);

// Sums the per-block FP64 partials (5 per block) in a fixed order: one block,
// each thread accumulates a strided subset, then a shared-memory tree.  The
// result does not depend on scheduling, so repeated runs agree bit for bit.
__global__ void __launch_bounds__(256) reduce_finish_kernel(const double* __restrict__ partials, uint32_t n_blocks,
                                                            double* __restrict__ out) {
    __shared__ double sm[256][5];
    double acc[5] = {0, 0, 0, 0, 0};
    for (uint32_t b = threadIdx.x; b < n_blocks; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < 5; k++) acc[k] += partials[(uint64_t)b * 5 + k];
#pragma unroll
    for (int k = 0; k < 5; k++) sm[threadIdx.x][k] = acc[k];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
#pragma unroll
            for (int k = 0; k < 5; k++) sm[threadIdx.x][k] += sm[threadIdx.x + s][k];
        __syncthreads();
    }
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 5; k++) out[k] = sm[0][k];
}

cudaError_t launch_reduce_finish(const double* partials, uint32_t n_blocks, double* out, cudaStream_t st) {
    reduce_finish_kernel<<<1, 256, 0, st>>>(partials, n_blocks, out);
    return cudaGetLastError();
}

}  // namespace bf
