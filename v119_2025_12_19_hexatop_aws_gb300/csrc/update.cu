// Density update between SIMP solves: the stress-ratio proposal, the update
// statistics, the culling of the weakest low-density elements and the hard
// projection of TopologyOptimization.update_density!
// (src/Optimization/TopOpt.jl:211-482), on the device with no host round trip
// between the passes.
//
//  propose   proposed_e = original_e (protected) or
//            max((l1_e / l1_allowable) / E, min_density)      TopOpt.jl:254-263
//  update    per unprotected element: raw = max(filtered, min_density),
//            |min(raw, max_density) - old| summed, raw > min_density counted;
//            the clamp to max_density, the active count (protected elements by
//            their original density) and the cull candidates
//            (min_density < rho < threshold)                   TopOpt.jl:369-447
//  select    the k = floor(active * max_culling_ratio) smallest candidates,
//            ties by element index (Julia's stable sort! of the candidate
//            list), by a radix select over the 64-bit key
//            (float bits of rho << 32 | index): six passes of 11-bit digits
//            from the top, each a histogram and a one-block prefix pick
//                                                              TopOpt.jl:449-460
//  finish    culled -> min_density, the "hard" projection rho > min_density
//            -> 1, protected elements back to their original density
//                                                              TopOpt.jl:462-481
//
// Every float operation the reference rounds is one rounded operation here
// (__fdiv_rn; min/max are exact), so densities, counts and the culled set are
// bit-identical to the reference's on the same filtered field; the mean change
// is a sum whose order the reference itself leaves to its thread count.
#include <cuda_runtime.h>

#include <algorithm>

#include "hexa_common.cuh"
#include "hexa_kernels.h"

namespace hexa {

namespace {

constexpr int kUpdBlocks = 152 * 4;
constexpr int kUpdThreads = 256;
constexpr int kDigitBits = 11;
constexpr int kBins = 1 << kDigitBits;

__device__ __forceinline__ bool is_candidate(float d, float min_d, float thr) { return d > min_d && d < thr; }

__device__ __forceinline__ unsigned long long cull_key(float d, long long e) {
  return ((unsigned long long)__float_as_uint(d) << 32) | (unsigned long long)e;
}

__global__ void propose_kernel(long long n, const float* __restrict__ l1, const uint8_t* __restrict__ prot,
                               const float* __restrict__ orig, float allow, float E, float min_d,
                               float* __restrict__ prop, UpdateState* __restrict__ s) {
  bool nan = false;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float v = l1[e];
    nan |= (v != v);
    prop[e] = (prot && prot[e]) ? orig[e] : fmaxf(__fdiv_rn(__fdiv_rn(v, allow), E), min_d);
  }
  if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) atomicOr(&s->nan_stress, 1);
}

// The update pass; per-block partial sums land in part[4 * blockIdx.x + ...]
// (change as FP64, three counts as unsigned 64-bit in the same double slots).
__global__ void __launch_bounds__(kUpdThreads) update_kernel(long long n, const float* __restrict__ old,
                                                             const float* __restrict__ src,
                                                             const uint8_t* __restrict__ prot,
                                                             const float* __restrict__ orig, float min_d,
                                                             float max_d, float thr, float* __restrict__ out,
                                                             double* __restrict__ part, UpdateState* __restrict__ s) {
  double change = 0.0;
  unsigned long long act1 = 0, act2 = 0, cand = 0;
  bool nan = false;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float f = src[e];
    nan |= (f != f);
    if (prot && prot[e]) {
      act2 += orig[e] > min_d;
      out[e] = old[e];  // restored to the original density at the end
      continue;
    }
    const float raw = fmaxf(f, min_d);
    change += (double)fabsf(fminf(raw, max_d) - old[e]);
    act1 += raw > min_d;
    const float d = fminf(raw, max_d);
    const bool live = d > min_d;
    act2 += live;
    cand += live && d < thr;
    out[e] = d;
  }
  if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) atomicOr(&s->nan_filtered, 1);
  __shared__ double sc[kUpdThreads / 32];
  __shared__ unsigned long long sa[3][kUpdThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    change += __shfl_xor_sync(0xffffffffu, change, o);
    act1 += __shfl_xor_sync(0xffffffffu, act1, o);
    act2 += __shfl_xor_sync(0xffffffffu, act2, o);
    cand += __shfl_xor_sync(0xffffffffu, cand, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) sc[w] = change, sa[0][w] = act1, sa[1][w] = act2, sa[2][w] = cand;
  __syncthreads();
  if (threadIdx.x == 0) {
    double c = 0.0;
    unsigned long long a = 0, b = 0, k = 0;
    for (int i = 0; i < kUpdThreads / 32; ++i) c += sc[i], a += sa[0][i], b += sa[1][i], k += sa[2][i];
    part[4 * blockIdx.x] = c;
    reinterpret_cast<unsigned long long*>(part)[4 * blockIdx.x + 1] = a;
    reinterpret_cast<unsigned long long*>(part)[4 * blockIdx.x + 2] = b;
    reinterpret_cast<unsigned long long*>(part)[4 * blockIdx.x + 3] = k;
  }
}

// One thread sums the partials in block order (deterministic) and fixes the
// culling mode: 0 none, 1 every candidate, 2 the k smallest keys.
__global__ void update_finalize_kernel(int nb, const double* __restrict__ part, float ratio,
                                       UpdateState* __restrict__ s) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double c = 0.0;
  unsigned long long a = 0, b = 0, k = 0;
  const unsigned long long* pu = reinterpret_cast<const unsigned long long*>(part);
  for (int i = 0; i < nb; ++i) c += part[4 * i], a += pu[4 * i + 1], b += pu[4 * i + 2], k += pu[4 * i + 3];
  s->change = c;
  s->active_updated = a;
  s->active = b;
  s->candidates = k;
  // Int * Float32 is a Float32 product in Julia, floored to Int
  const unsigned long long allowed = (unsigned long long)floorf(__fmul_rn(__ull2float_rn(b), ratio));
  s->allowed = allowed;
  s->mode = (k <= allowed) ? 1 : (allowed > 0 ? 2 : 0);
  s->culled = (k <= allowed) ? k : allowed;
  s->prefix = 0ull;
  s->remaining = allowed;
  s->mean_change = a > 0 ? __fdiv_rn((float)c, __ull2float_rn(a)) : 0.0f;
}

__device__ __forceinline__ void digit_span(int pass, int* shift, int* width) {
  // passes from the top: bits [53,64), [42,53), [31,42), [20,31), [9,20), [0,9)
  const int top = 64 - kDigitBits * pass;
  *width = top >= kDigitBits ? kDigitBits : top;
  *shift = top - *width;
}

__global__ void __launch_bounds__(kUpdThreads) select_hist_kernel(long long n, const float* __restrict__ d,
                                                                  const uint8_t* __restrict__ prot, float min_d,
                                                                  float thr, int pass,
                                                                  const UpdateState* __restrict__ s,
                                                                  unsigned long long* __restrict__ hist) {
  if (s->mode != 2) return;
  __shared__ unsigned int h[kBins];
  for (int i = threadIdx.x; i < kBins; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  int shift, width;
  digit_span(pass, &shift, &width);
  const int above = shift + width;  // bits at and above this position are fixed by the prefix
  const unsigned long long prefix = s->prefix;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    if (prot && prot[e]) continue;
    const float v = d[e];
    if (!is_candidate(v, min_d, thr)) continue;
    const unsigned long long key = cull_key(v, e);
    if (above < 64 && (key >> above) != (prefix >> above)) continue;
    atomicAdd(&h[(key >> shift) & ((1u << width) - 1u)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kBins; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], (unsigned long long)h[i]);
}

// One block of kBins / 2 threads: thread t owns bins 2t and 2t + 1; an
// exclusive scan finds the digit holding the remaining-th smallest key.
__global__ void __launch_bounds__(kBins / 2) select_pick_kernel(int pass, UpdateState* __restrict__ s,
                                                                unsigned long long* __restrict__ hist) {
  if (s->mode != 2) return;
  constexpr int NT = kBins / 2;
  __shared__ unsigned long long wsum[NT / 32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const unsigned long long c0 = hist[2 * t], c1 = hist[2 * t + 1];
  unsigned long long incl = c0 + c1;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    unsigned long long v = lane < NT / 32 ? wsum[lane] : 0ull;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    if (lane < NT / 32) wsum[lane] = v;  // inclusive over warps
  }
  __syncthreads();
  const unsigned long long excl = incl - (c0 + c1) + (w > 0 ? wsum[w - 1] : 0ull);
  const unsigned long long rem = s->remaining;
  int shift, width;
  digit_span(pass, &shift, &width);
  __syncthreads();
  if (excl < rem && rem <= excl + c0) {
    s->prefix |= (unsigned long long)(2 * t) << shift;
    s->remaining = rem - excl;
  } else if (excl + c0 < rem && rem <= excl + c0 + c1) {
    s->prefix |= (unsigned long long)(2 * t + 1) << shift;
    s->remaining = rem - excl - c0;
  }
  hist[2 * t] = 0ull;
  hist[2 * t + 1] = 0ull;
}

__global__ void finish_kernel(long long n, float* __restrict__ d, const uint8_t* __restrict__ prot,
                              const float* __restrict__ orig, float min_d, float thr, int hard,
                              const UpdateState* __restrict__ s) {
  const int mode = s->mode;
  const unsigned long long kth = s->prefix;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    if (prot && prot[e]) {
      d[e] = orig[e];
      continue;
    }
    float v = d[e];
    if (is_candidate(v, min_d, thr) && (mode == 1 || (mode == 2 && cull_key(v, e) <= kth))) v = min_d;
    if (hard && v > min_d) v = 1.0f;
    d[e] = v;
  }
}

int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16)); }

}  // namespace

void launch_propose(long long n, const float* l1, const uint8_t* prot, const float* orig, float allow, float E,
                    float min_d, float* prop, UpdateState* s, cudaStream_t st) {
  propose_kernel<<<grid_for(n), 256, 0, st>>>(n, l1, prot, orig, allow, E, min_d, prop, s);
}

int launch_update_cull(long long n, const float* old, const float* src, const uint8_t* prot, const float* orig,
                       float min_d, float max_d, float thr, float ratio, int hard, float* out, double* part,
                       unsigned long long* hist, UpdateState* s, cudaStream_t st) {
  int launches = 0;
  cudaMemsetAsync(hist, 0, kBins * sizeof(unsigned long long), st);
  update_kernel<<<kUpdBlocks, kUpdThreads, 0, st>>>(n, old, src, prot, orig, min_d, max_d, thr, out, part, s);
  update_finalize_kernel<<<1, 32, 0, st>>>(kUpdBlocks, part, ratio, s);
  launches += 2;
  for (int pass = 0; pass < (64 + kDigitBits - 1) / kDigitBits; ++pass) {
    select_hist_kernel<<<grid_for(n), kUpdThreads, 0, st>>>(n, out, prot, min_d, thr, pass, s, hist);
    select_pick_kernel<<<1, kBins / 2, 0, st>>>(pass, s, hist);
    launches += 2;
  }
  finish_kernel<<<grid_for(n), 256, 0, st>>>(n, out, prot, orig, min_d, thr, hard, s);
  return launches + 1;
}

size_t update_partials_doubles() { return 4 * (size_t)kUpdBlocks; }
int update_hist_bins() { return kBins; }

}  // namespace hexa
