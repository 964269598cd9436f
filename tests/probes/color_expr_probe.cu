// Probe for tests/test_gpu_color.py: evaluates the reference's colour
// conversion expressions (src/color_space.cuh:18-21) exactly as written,
// compiled by nvcc with its default flags, so the test can see which
// floating-point evaluation order the compiler gives them.  One thread per
// pixel, grid sized from n on the host; every index is checked against n.
#include <cuda_runtime.h>

__global__ void probe_ycbcr(const uchar4* in, uchar4* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uchar4 val = in[i];
  out[i] = make_uchar4(val.x * 0.299 + 0.587 * val.y + 0.114 * val.z,
                       128 - val.x * 0.168736 - 0.331264 * val.y + 0.5 * val.z,
                       128 + val.x * 0.5 - 0.418688 * val.y - 0.081312 * val.z,
                       val.w);
}

extern "C" int probe_run(const void* h_in, void* h_out, int n) {
  uchar4 *d_in = nullptr, *d_out = nullptr;
  const size_t bytes = (size_t)n * sizeof(uchar4);
  if (cudaMalloc(&d_in, bytes) != cudaSuccess) return 1;
  if (cudaMalloc(&d_out, bytes) != cudaSuccess) { cudaFree(d_in); return 2; }
  int rc = 0;
  if (cudaMemcpy(d_in, h_in, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = 3;
  if (!rc) {
    const int threads = 256, blocks = (n + threads - 1) / threads;
    probe_ycbcr<<<blocks, threads>>>(d_in, d_out, n);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = 4;
  }
  if (!rc && cudaMemcpy(h_out, d_out, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 5;
  cudaFree(d_in);
  cudaFree(d_out);
  return rc;
}
