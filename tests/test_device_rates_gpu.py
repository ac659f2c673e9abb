"""The device rates the kernels' design rests on, measured on the GPU that runs the tests.

A small CUDA program (compiled here with nvcc for sm_103a) times, over all SMs:
  - FP64 and FP32 fused multiply-adds (four independent chains per thread);
  - FP64 -> FP32 conversions;
  - the cycles a thread spends issuing one cp.async.bulk copy into shared memory.
The test prints the figures (run with -s) and checks what the design relies on: FP64
arithmetic runs at a small fraction of the FP32 rate on this part, and a bulk copy keeps its
issuing thread for hundreds of cycles.
"""
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

SRC = r"""
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
constexpr int IT = 2048;
__global__ void f64fma(double *out, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < IT; i++) { x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b); }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
__global__ void f32fma(float *out, float a, float b) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < IT; i++) { x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b); }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
// four FP64 -> FP32 conversions of four distinct values per iteration (integer ops make
// the values; they cost far less than the conversions)
__global__ void d2f(float *out, const double *in) {
  float x0 = 0, x1 = 0, x2 = 0, x3 = 0;
  long long b = __double_as_longlong(in[threadIdx.x & 31]);
  for (int i = 0; i < IT; i++) {
    x0 += (float)__longlong_as_double(b);
    x1 += (float)__longlong_as_double(b ^ (1ll << 40));
    x2 += (float)__longlong_as_double(b ^ (2ll << 40));
    x3 += (float)__longlong_as_double(b ^ (3ll << 40));
    b ^= 1ll << 36;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
__device__ __forceinline__ uint32_t sa(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// thread 0 of each CTA issues K bulk copies of S bytes per round, then waits (bounded)
__global__ void bulk(const char *src, size_t bytes, int K, int S, int rounds, unsigned long long *out) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(&bar)), "r"(1) : "memory");
  __syncthreads();
  unsigned long long ti = 0;
  uint32_t ph = 0;
  for (int r = 0; r < rounds; r++) {
    if (threadIdx.x == 0) {
      const unsigned long long t0 = clock64();
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(&bar)), "r"(K * S) : "memory");
      for (int c = 0; c < K; c++) {
        const size_t off = (((size_t)blockIdx.x * rounds + r) * K + c) * (size_t)S % (bytes - S);
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(sa(sm + c * S)), "l"(src + (off & ~(size_t)15)), "r"(S), "r"(sa(&bar)) : "memory");
      }
      ti += clock64() - t0;
      uint32_t ok = 0;
      for (long long g = 0; !ok && g < 100000000ll; g++)
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok) : "r"(sa(&bar)), "r"(ph) : "memory");
    }
    ph ^= 1;
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(out, ti);
}
int main() {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int blocks = sms * 8, threads = 256;
  const size_t n = (size_t)blocks * threads;
  double *od, *in; float *of;
  cudaMalloc(&od, n * 8); cudaMalloc(&of, n * 4); cudaMalloc(&in, 256);
  double h[32]; for (int i = 0; i < 32; i++) h[i] = -0.065 + 1e-3 * i;
  cudaMemcpy(in, h, 256, cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  auto rate = [&](auto launch) {  // operations per second
    launch(); cudaDeviceSynchronize();
    cudaEventRecord(e0); for (int r = 0; r < 3; r++) launch(); cudaEventRecord(e1); cudaEventSynchronize(e1);
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    return 3.0 * n * IT * 4 / (ms * 1e-3);
  };
  const double r64 = rate([&] { f64fma<<<blocks, threads>>>(od, 0.999, 1e-3); });
  const double r32 = rate([&] { f32fma<<<blocks, threads>>>(of, 0.999f, 1e-3f); });
  const double rcv = rate([&] { d2f<<<blocks, threads>>>(of, in); });
  const size_t bytes = (size_t)1 << 30;
  char *src; cudaMalloc(&src, bytes); cudaMemset(src, 1, bytes);
  unsigned long long *cyc; cudaMalloc(&cyc, 8); cudaMemset(cyc, 0, 8);
  cudaFuncSetAttribute(bulk, cudaFuncAttributeMaxDynamicSharedMemorySize, 48 * 1024);
  const int K = 8, S = 2048, rounds = 100, grid = sms * 4;
  bulk<<<grid, 256, 48 * 1024>>>(src, bytes, K, S, rounds, cyc);
  unsigned long long c = 0; cudaMemcpy(&c, cyc, 8, cudaMemcpyDeviceToHost);
  const cudaError_t err = cudaDeviceSynchronize();
  printf("%.6e %.6e %.6e %.3f %d %s\n", r64, r32, rcv, (double)c / ((double)grid * rounds * K), sms,
         err == cudaSuccess ? "ok" : cudaGetErrorString(err));
  return err == cudaSuccess ? 0 : 1;
}
"""


def test_device_rates(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "rates.cu"
    src.write_text(SRC)
    exe = tmp_path / "rates"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", str(src), "-o",
                    str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    r64, r32, rcv, issue, sms = float(out[0]), float(out[1]), float(out[2]), float(out[3]), int(out[4])
    assert out[5] == "ok"
    print(f"\nFP64 FMA {r64 * 2 / 1e12:.2f} TFLOP/s ({r64 / sms / 2.07e9:.2f} per clock per SM at "
          f"2.07 GHz); FP32 FMA {r32 * 2 / 1e12:.1f} TFLOP/s ({r32 / sms / 2.07e9:.1f}); FP64->FP32 "
          f"conversions {rcv / 1e9:.0f} G/s ({rcv / sms / 2.07e9:.2f}); bulk copy issue "
          f"{issue:.0f} cycles per copy")
    assert r32 > 20 * r64       # FP64 arithmetic is far below FP32 on this part
    assert 50 < issue < 5000    # a bulk copy keeps its issuing thread for hundreds of cycles


COOP_SRC = r"""
#include <cstdio>
#include <cooperative_groups.h>
#include <cuda_runtime.h>
namespace cg = cooperative_groups;
// spins for a fixed number of clock cycles (waits on nothing else), then one grid sync
__global__ void spin(long long cycles, int *out) {
  cg::grid_group g = cg::this_grid();
  const long long t0 = clock64();
  while (clock64() - t0 < cycles) {}
  g.sync();
  if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(out, 1);
}
int main() {
  int *out; cudaMalloc(&out, 4); cudaMemset(out, 0, 4);
  cudaStream_t s[4];
  for (int i = 0; i < 4; i++) cudaStreamCreateWithFlags(&s[i], cudaStreamNonBlocking);
  long long cyc = 20000000;  // ~10 ms at 2 GHz
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float t[2];
  for (int k = 0; k < 2; k++) {
    const int n = k == 0 ? 1 : 4;
    cudaDeviceSynchronize();
    cudaEventRecord(e0, 0);
    cudaDeviceSynchronize();
    for (int i = 0; i < n; i++) {
      void *args[] = {&cyc, &out};
      cudaLaunchCooperativeKernel((void *)spin, 20, 256, args, 0, s[i]);
    }
    cudaDeviceSynchronize();
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&t[k], e0, e1);
  }
  const cudaError_t err = cudaDeviceSynchronize();
  printf("%.3f %.3f %s\n", t[0], t[1], err == cudaSuccess ? "ok" : cudaGetErrorString(err));
  return err == cudaSuccess ? 0 : 1;
}
"""


def test_cooperative_launches_overlap(tmp_path):
    """Cooperative launches on different streams run at the same time (the server steps
    each wide implicit request as a cooperative launch on its batch's own stream): four
    20-CTA kernels that each spin ~10 ms take about as long as one."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src = tmp_path / "coop.cu"
    src.write_text(COOP_SRC)
    exe = tmp_path / "coop"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", str(src), "-o",
                    str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    one, four = float(out[0]), float(out[1])
    assert out[2] == "ok"
    print(f"\none cooperative kernel {one:.2f} ms; four on four streams {four:.2f} ms")
    assert four < 1.5 * one
