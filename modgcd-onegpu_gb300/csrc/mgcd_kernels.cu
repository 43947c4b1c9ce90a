// mgcd_kernels.cu -- the modular GCD kernels for sm_103a.
//
// One gcd pair is processed by one CTA (batched, persistent kernel pulling pairs from a
// size-ordered queue) or, when its moduli do not fit one CTA, by a cooperative grid.
// Stages, with the reference's labels (GmpCudaDevice-getGcdKernel.cu:342-444):
//   MGCD2  residues of u and v for every modulus: limb tiles staged in shared memory,
//          Montgomery Horner per modulus (z <- REDC(z * 2^64 mod q + limb));
//   MGCD3  reduction loop: per modulus only t = u/v mod q is kept; each iteration picks
//          the pivot (p, b) = argmin of the reference's key (|t|, q - sign) with warp
//          redux.sync minima and one barrier, then updates t' = p / (t - b) (one modular
//          inverse per update; the reference needs two) and records (p, b);
//   replay the surviving moduli rebuild u mod q by applying the recorded (p, b) sequence
//          to their initial residues projectively (three Montgomery products per step, no
//          inverse) and dividing out the accumulated scale once;
//   MGCD4  recovery: signed mixed-radix digits, next digit from the lowest-indexed
//          modulus with a nonzero value, exactly as the reference selects it.
// The (p, b) sequence and the digits are identical to the reference algorithm's.
#include <cstdint>
#include <cuda_runtime.h>

#include "mgcd_device.cuh"
#include "mgcd_internal.h"
#include "mgcd_pair.cuh"

namespace mgcd {

// Persistent batched kernel: each CTA repeatedly takes the next pair of the queue (pairs
// ordered largest first) and computes its gcd alone.
template <int T>
__global__ void __launch_bounds__(T) batch_kernel(const BatchArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ RedSmem rs;
  __shared__ uint32_t next;
  uint32_t* st = smem;
  uint32_t* acc2 = smem + a.nq_max;
  uint32_t* chunk = acc2 + a.nq_max;
  uint32_t* scr = a.scratch + (size_t)blockIdx.x * a.scratch_words;
  uint32_t* u0 = scr;
  uint32_t* v0 = scr + a.nq_max;
  int2* hist = reinterpret_cast<int2*>(scr + 2 * (size_t)a.nq_max);
  for (;;) {
    if (threadIdx.x == 0) next = atomicAdd(a.queue, 1u);
    __syncthreads();
    const uint32_t k = next;
    __syncthreads();
    if (k >= a.npairs) break;
    const uint32_t pi = a.order[k];
    const PairDesc d = a.pairs[pi];
    run_pair<T, false>(a.limbs, d, a.mods, a.L, 0u, d.nq, st, acc2, chunk, rs, u0, v0, hist, nullptr,
                       a.digits, a.count + pi, a.iters + pi, a.status + pi);
    __syncthreads();
  }
}

// One pair over a cooperative grid of GRID_THREADS-thread CTAs; CTA c owns moduli
// [c * per_cta, min(nq, (c + 1) * per_cta)).
__global__ void __launch_bounds__(GRID_THREADS) grid_kernel(const GridArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ RedSmem rs;
  const uint32_t nq = a.pair.nq;
  const uint32_t j0 = blockIdx.x * a.per_cta;
  const uint32_t nloc = j0 >= nq ? 0u : (nq - j0 < a.per_cta ? nq - j0 : a.per_cta);
  uint32_t* st = smem;
  uint32_t* acc2 = smem + a.per_cta;
  uint32_t* chunk = acc2 + a.per_cta;
  uint32_t* u0 = a.scratch + j0;
  uint32_t* v0 = a.scratch + nq + j0;
  int2* hist = reinterpret_cast<int2*>(a.scratch + 2 * (size_t)nq);
  run_pair<GRID_THREADS, true>(a.limbs, a.pair, a.mods, a.L, j0, nloc, st, acc2, chunk, rs, u0, v0, hist,
                               a.sync, a.digits, a.count, a.iters, a.status);
}

// Integer-pipe microbenchmark: eight independent IMAD chains per thread.
__global__ void __launch_bounds__(256) int_peak_kernel(uint32_t* out, int iters)
{
  uint32_t a0 = threadIdx.x, a1 = a0 ^ 1u, a2 = a0 ^ 2u, a3 = a0 ^ 3u;
  uint32_t a4 = a0 ^ 4u, a5 = a0 ^ 5u, a6 = a0 ^ 6u, a7 = a0 ^ 7u;
  const uint32_t c = blockIdx.x | 1u;
  uint32_t m = 0x9E3779B9u ^ (uint32_t)iters;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
    a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
    a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
  }
  if ((a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7) == 0x2545F491u) out[0] = 1u;
}

cudaError_t launch_int_peak(uint32_t* out, int blocks, int iters, cudaStream_t s)
{
  int_peak_kernel<<<blocks, 256, 0, s>>>(out, iters);
  return cudaGetLastError();
}

// ------------------------------------------------------------------- launchers ----

size_t batch_smem_bytes(int /*threads*/, uint32_t nq_max)
{
  return sizeof(uint32_t) * (2 * (size_t)nq_max + CHUNK);
}

template <int T>
static const void* batch_fn()
{
  return reinterpret_cast<const void*>(&batch_kernel<T>);
}

static const void* batch_fn_for(int threads)
{
  switch (threads) {
    case 256: return batch_fn<256>();
    case 512: return batch_fn<512>();
    case 1024: return batch_fn<1024>();
    default: return nullptr;
  }
}

cudaError_t batch_max_blocks_per_sm(int threads, size_t smem, int* blocks)
{
  const void* fn = batch_fn_for(threads);
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, threads, smem);
}

cudaError_t launch_batch(const BatchArgs& a, int threads, int grid, size_t smem, cudaStream_t s)
{
  const void* fn = batch_fn_for(threads);
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<BatchArgs*>(&a)};
  return cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, smem, s);
}

size_t grid_smem_bytes(uint32_t per_cta)
{
  return sizeof(uint32_t) * (2 * (size_t)per_cta + CHUNK);
}

cudaError_t grid_max_blocks_per_sm(size_t smem, int* blocks)
{
  const void* fn = reinterpret_cast<const void*>(&grid_kernel);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, GRID_THREADS, smem);
}

cudaError_t launch_grid(const GridArgs& a, int grid, size_t smem, cudaStream_t s)
{
  const void* fn = reinterpret_cast<const void*>(&grid_kernel);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<GridArgs*>(&a)};
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(GRID_THREADS), args, smem, s);
}

}  // namespace mgcd
