// hz_l2_probe.cu -- L2 read bandwidth probe used by the benchmark's roofline.
//
// The search kernel's working set (BVH nodes and triangles near the cells in
// flight) is largely L2 resident, so its algorithmic bytes are also compared
// with the L2 read bandwidth of this GPU. This probe streams a caller-provided
// device buffer that fits in L2 (e.g. 32 MiB) `reps` times with 16-byte loads
// that bypass L1 (ld.global.cg) from a grid of every SM, after one untimed
// pass that makes it resident, and reports the time of the timed passes.
// Not part of the horizon library's interface.
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(512) k_l2_read(const float4* __restrict__ buf, long long n,
                                                 int reps, unsigned* __restrict__ sink) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long start = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned acc = 0u;
  for (int r = 0; r < reps; r++) {
    for (long long i = start; i < n; i += stride) {
      const float4 v = __ldcg(buf + i);
      acc ^= __float_as_uint(v.x) ^ __float_as_uint(v.y) ^ __float_as_uint(v.z) ^
             __float_as_uint(v.w);
    }
  }
  if (acc == 0x9E3779B9u) sink[0] = acc;  // keeps the loads; practically never taken
}

}  // namespace

// Returns 0 on success; *ms = duration of `reps` passes over `bytes` bytes.
extern "C" int hz_probe_l2_read(const void* buf, long long bytes, int reps, void* sink,
                                void* stream, float* ms) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 1;
  const long long n = bytes / 16;
  if (n <= 0 || reps <= 0) return 2;
  const unsigned blocks = (unsigned)sms * 4u;
  const float4* p = static_cast<const float4*>(buf);
  unsigned* k = static_cast<unsigned*>(sink);
  k_l2_read<<<blocks, 512, 0, s>>>(p, n, 1, k);  // make resident
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  k_l2_read<<<blocks, 512, 0, s>>>(p, n, reps, k);
  cudaEventRecord(e1, s);
  const cudaError_t e = cudaEventSynchronize(e1);
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e == cudaSuccess && cudaGetLastError() == cudaSuccess ? 0 : 3;
}
