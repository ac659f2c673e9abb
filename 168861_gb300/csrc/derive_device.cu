// Parameter pipeline on the device for many trees at once (nrt_derive_batch).
//
// Each tree is one CTA.  Its threads take the tree's elements 256 at a time and run the
// per-element pipeline of derive_elem.h (the same code nrt_derive runs on the host); HH
// elements get their place in the tree's HH list from a ballot prefix within the chunk
// plus the count of earlier chunks, and the critical time step is the CTA's minimum over
// elements 1 .. n-2 (src/init.cpp:160-174).  The trees of a batch arrive packed back to
// back, so one copy in and one copy out serve all of them.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "derive_elem.h"
#include "nrt_internal.h"
#include "pdl.cuh"

namespace nrt {

namespace {

constexpr int kDThreads = 256;

struct DeriveArgs {
  const int64_t *off;       // [count + 1] element offsets
  const int64_t *hh_off;    // [count + 1] HH offsets
  const int32_t *kind;      // ispec row 0, all trees
  const double *dspec;      // [12][total]
  const int32_t *myelin;    // [count]
  const double *e_max;      // [count]
  double *eparam;           // [6][total]
  int32_t *hh_elem;         // [hh_total] local element indices
  double *hparam;           // [12][hh_total]
  double *dT_crit;          // [count]
  int64_t total, hh_total;
};

__global__ void __launch_bounds__(kDThreads) derive_trees(DeriveArgs a) {
  __shared__ int warp_cnt[kDThreads / 32];
  __shared__ double warp_min[kDThreads / 32];
  const int t = blockIdx.x;
  const int64_t o = a.off[t], n = a.off[t + 1] - o, h0 = a.hh_off[t];
  const int64_t T = a.total, H = a.hh_total;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int my = a.myelin[t];
  const double emax = a.e_max[t];
  double tmin = INFINITY;
  int64_t before = 0;  // HH elements in earlier chunks
  for (int64_t c0 = 0; c0 < n; c0 += kDThreads) {
    const int64_t jl = c0 + threadIdx.x;
    const bool ok = jl < n;
    const int64_t i = o + jl;
    const bool hh = ok && a.kind[i] == 1;
    const unsigned bal = __ballot_sync(0xffffffffu, hh);
    if (lane == 0) warp_cnt[w] = __popc(bal);
    __syncthreads();
    int wbase = 0, chunk = 0;
    for (int q = 0; q < kDThreads / 32; q++) {
      if (q < w) wbase += warp_cnt[q];
      chunk += warp_cnt[q];
    }
    const int64_t pos = before + wbase + __popc(bal & ((1u << lane) - 1u));
    if (ok) {
      nrt_param::ElemIn in;
      in.kind = a.kind[i];
      in.dX0 = a.dspec[i];
      in.diam0 = a.dspec[T + i];
      in.eps = a.dspec[2 * T + i];
      in.ro_a = a.dspec[4 * T + i];
      in.ro_m = a.dspec[5 * T + i];
      in.per_m = a.dspec[6 * T + i];
      in.th = a.dspec[7 * T + i];
      in.rest = a.dspec[8 * T + i];
      in.sna = a.dspec[9 * T + i];
      in.sk = a.dspec[10 * T + i];
      in.sl = a.dspec[11 * T + i];
      double ep[6], hp[12];
      nrt_param::derive_element(in, my, emax, ep, hp);
#pragma unroll
      for (int q = 0; q < 6; q++) a.eparam[q * T + i] = ep[q];
      if (hh) {
        a.hh_elem[h0 + pos] = (int32_t)jl;
#pragma unroll
        for (int q = 0; q < 12; q++) a.hparam[q * H + h0 + pos] = hp[q];
      }
      // the reference's selection (src/init.cpp:160-174): the smallest over 1 .. n-2
      if (jl >= 1 && jl <= n - 2 && ep[5] < tmin) tmin = ep[5];
    }
    before += chunk;
    __syncthreads();  // warp_cnt reused by the next chunk
  }
  for (int s = 16; s > 0; s >>= 1) tmin = fmin(tmin, __shfl_down_sync(0xffffffffu, tmin, s));
  if (lane == 0) warp_min[w] = tmin;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = warp_min[0];
    for (int q = 1; q < kDThreads / 32; q++) m = fmin(m, warp_min[q]);
    a.dT_crit[t] = m;
  }
}

// Device buffers of one call, freed on every path.
struct DevBufs {
  std::vector<void *> p;
  ~DevBufs() {
    for (void *q : p) cudaFree(q);
  }
  template <class X>
  X *take(size_t count) {
    void *q = nullptr;
    if (cudaMalloc(&q, sizeof(X) * std::max<size_t>(count, 1)) != cudaSuccess) return nullptr;
    p.push_back(q);
    return (X *)q;
  }
};

}  // namespace

}  // namespace nrt

extern "C" int nrt_derive_batch(int32_t count, const int64_t *offsets, const int32_t *ispec,
                                const double *dspec, const int32_t *myelin, const double *e_max,
                                double *eparam, int32_t *hh_elem, double *hparam,
                                int64_t *hh_offsets, double *dT_crit) {
  return nrt::guarded([&]() -> int {
    using namespace nrt;
    if (count < 1 || !offsets || !ispec || !dspec || !myelin || !e_max || !eparam ||
        !hh_offsets || !dT_crit) {
      set_error("null argument or count < 1");
      return NRT_EINVAL;
    }
    if (offsets[0] != 0) {
      set_error("offsets[0] must be 0");
      return NRT_EINVAL;
    }
    for (int32_t t = 0; t < count; t++)
      if (offsets[t + 1] - offsets[t] < 4) {
        set_error("tree " + std::to_string(t) + " has fewer than 4 elements");
        return NRT_EINVAL;
      }
    const int64_t T = offsets[count];
    // HH counts per tree (the kind row is on the host already)
    std::vector<int64_t> cnt(count, 0);
    parallel_for(count, [&](int64_t t) {
      int64_t c = 0;
      for (int64_t i = offsets[t]; i < offsets[t + 1]; i++) c += ispec[i] == 1;
      cnt[t] = c;
    });
    hh_offsets[0] = 0;
    for (int32_t t = 0; t < count; t++) hh_offsets[t + 1] = hh_offsets[t] + cnt[t];
    const int64_t H = hh_offsets[count];
    if (H > 0 && (!hh_elem || !hparam)) {
      set_error("null HH output");
      return NRT_EINVAL;
    }
    cudaStream_t st;
    NRT_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{st};
    DevBufs d;
    int64_t *d_off = d.take<int64_t>(count + 1), *d_hoff = d.take<int64_t>(count + 1);
    int32_t *d_kind = d.take<int32_t>(T), *d_my = d.take<int32_t>(count),
            *d_hh = d.take<int32_t>(H);
    double *d_ds = d.take<double>(12 * (size_t)T), *d_em = d.take<double>(count),
           *d_ep = d.take<double>(6 * (size_t)T), *d_hp = d.take<double>(12 * (size_t)H),
           *d_dt = d.take<double>(count);
    if (!d_off || !d_hoff || !d_kind || !d_my || !d_hh || !d_ds || !d_em || !d_ep || !d_hp ||
        !d_dt) {
      cudaGetLastError();
      set_error("device allocation for the derivation");
      return NRT_ENOMEM;
    }
    NRT_CUDA(cudaMemcpyAsync(d_off, offsets, 8 * (size_t)(count + 1), cudaMemcpyHostToDevice, st));
    NRT_CUDA(cudaMemcpyAsync(d_hoff, hh_offsets, 8 * (size_t)(count + 1), cudaMemcpyHostToDevice, st));
    NRT_CUDA(cudaMemcpyAsync(d_kind, ispec, 4 * (size_t)T, cudaMemcpyHostToDevice, st));
    NRT_CUDA(cudaMemcpyAsync(d_my, myelin, 4 * (size_t)count, cudaMemcpyHostToDevice, st));
    NRT_CUDA(cudaMemcpyAsync(d_ds, dspec, 8 * 12 * (size_t)T, cudaMemcpyHostToDevice, st));
    NRT_CUDA(cudaMemcpyAsync(d_em, e_max, 8 * (size_t)count, cudaMemcpyHostToDevice, st));
    DeriveArgs a{d_off, d_hoff, d_kind, d_ds, d_my, d_em, d_ep, d_hh, d_hp, d_dt, T, H};
    derive_trees<<<count, kDThreads, 0, st>>>(a);
    count_launch_on(st);
    NRT_CUDA(cudaGetLastError());
    NRT_CUDA(cudaMemcpyAsync(eparam, d_ep, 8 * 6 * (size_t)T, cudaMemcpyDeviceToHost, st));
    if (H > 0) {
      NRT_CUDA(cudaMemcpyAsync(hh_elem, d_hh, 4 * (size_t)H, cudaMemcpyDeviceToHost, st));
      NRT_CUDA(cudaMemcpyAsync(hparam, d_hp, 8 * 12 * (size_t)H, cudaMemcpyDeviceToHost, st));
    }
    NRT_CUDA(cudaMemcpyAsync(dT_crit, d_dt, 8 * (size_t)count, cudaMemcpyDeviceToHost, st));
    NRT_CUDA(cudaStreamSynchronize(st));
    return NRT_OK;
  });
}
