// Ahead-of-time sm_103a kernels that do not depend on a rule set: grid digests and
// material histograms, used to check full-size worlds on the device without copying
// them out (order-independent digest; per-material counts for conservation checks).
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

__device__ __forceinline__ unsigned long long se_mix64(unsigned long long z) {
  // splitmix64 finaliser
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// digest = sum over cells of mix64(index * 2^32 + value)  (mod 2^64)
__global__ void __launch_bounds__(256) se_digest_kernel(const uint32_t* __restrict__ g, unsigned long long n,
                                                        unsigned long long* __restrict__ out) {
  unsigned long long acc = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    acc += se_mix64((i << 32) | g[i]);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ unsigned long long part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
    atomicAdd(out, s);
  }
}

// counts[min(value, nbins-1)] += 1
__global__ void __launch_bounds__(256) se_histogram_kernel(const uint32_t* __restrict__ g, unsigned long long n,
                                                           int nbins, unsigned long long* __restrict__ counts) {
  __shared__ unsigned int local[257];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) local[i] = 0;
  __syncthreads();
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t v = g[i];
    atomicAdd(&local[v < (uint32_t)nbins ? v : (uint32_t)(nbins - 1)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (local[i]) atomicAdd(&counts[i], (unsigned long long)local[i]);
}

}  // namespace

namespace se::rt {

cudaError_t grid_digest(const uint32_t* g, unsigned long long n, unsigned long long* d_out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  se_digest_kernel<<<sms * 8, 256, 0, s>>>(g, n, d_out);
  return cudaGetLastError();
}

cudaError_t grid_histogram(const uint32_t* g, unsigned long long n, int nbins, unsigned long long* d_counts,
                           cudaStream_t s) {
  if (nbins < 1 || nbins > 257) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(d_counts, 0, sizeof(unsigned long long) * (size_t)nbins, s);
  if (e != cudaSuccess) return e;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  se_histogram_kernel<<<sms * 4, 256, 0, s>>>(g, n, nbins, d_counts);
  return cudaGetLastError();
}

}  // namespace se::rt
