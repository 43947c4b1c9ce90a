// mgcd_noalloc.cu -- mgcd_gcd_digits_noalloc: the gcd of one pair without any allocation.
//
// Who needs it: code that may not call cudaMalloc at the point where it wants a gcd -- a
// real-time or callback context that must not block on the allocator or risk its failure,
// or an application whose device memory is budgeted and owned by its own pool, so that a
// library allocating behind its back would break that budget.  Such a caller brings its own
// device buffers for the operands and the results; the working memory this kernel needs
// besides them (each modulus's initial residues and the pivot history of the reduction
// loop) lives in the file-scope device array below, sized for the largest pair this entry
// point accepts.
//
// Limits and rules:
//   - 32-bit moduli only, at most NA_MAX_NQ = 4,096 moduli: operands up to about 38,000
//     bits.  Larger operands are rejected before anything is launched.
//   - The scratch array (64 KiB) and the moduli table (64 KiB) are static device memory:
//     every GPU that loads this library holds them until the process exits.
//   - The first call in a CUDA context (per device, and again after a device reset) sets it
//     up: looks up the arrays' device addresses and copies the moduli table in, a
//     synchronous copy.  Make that first call before any stream capture begins.
//   - Every call shares the one scratch array, which keeps the last call's contents.  The
//     kernel writes every scratch word it later reads within the same call, so nothing has
//     to start at zero.  Calls whose kernels overlap on the GPU (other streams, other host
//     threads) race on the scratch array: serialise them.
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/modgcd.h"
#include "mgcd_moduli.h"
#include "mgcd_pair.cuh"

namespace mgcd {
namespace {

constexpr uint32_t NA_MAX_NQ = 4096;
constexpr int NA_THREADS = 1024;
constexpr int NA_L = 32;
constexpr size_t NA_SCRATCH_WORDS = 4 * (size_t)NA_MAX_NQ;   // u0, v0, then (p, b) history
constexpr int NA_MAX_DEVICES = 64;

static __device__ __align__(256) uint32_t g_na_scratch[NA_SCRATCH_WORDS];
static __device__ __align__(256) ModConst g_na_mods[NA_MAX_NQ];

struct NaArgs {
  const uint32_t* limbs;     // u at limbs[0 .. u_len), v at limbs[u_len .. u_len + v_len)
  uint32_t u_len, v_len;
  uint32_t* scratch;         // device address of g_na_scratch
  const ModConst* mods;      // device address of g_na_mods
  uint32_t thr[NA_MAX_NQ / 256];  // thr[k]: fewest bits for which more than 256*(k+1) moduli are needed
  mgcd_pair* digits;
  uint32_t* count;
  int32_t* status;           // receives an MGCD_* code
};

__global__ void __launch_bounds__(NA_THREADS) noalloc_kernel(const NaArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ RedSmem rs;
  __shared__ PairDesc d;
  __shared__ int32_t pre;
  __shared__ uint32_t iters;
  if (threadIdx.x == 0) {
    uint32_t ul = a.u_len, vl = a.v_len;
    const uint32_t* U = a.limbs;
    const uint32_t* V = a.limbs + a.u_len;
    while (ul && U[ul - 1] == 0u) --ul;
    while (vl && V[vl - 1] == 0u) --vl;
    pre = MGCD_OK;
    if (ul == 0u || vl == 0u) {
      pre = MGCD_ERR_INVALID_ARG;
    } else {
      int c = (ul > vl) - (ul < vl);
      for (uint32_t i = ul; c == 0 && i-- > 0;) c = (U[i] > V[i]) - (U[i] < V[i]);
      if (c >= 0) { d.u_off = 0; d.u_len = ul; d.v_off = a.u_len; d.v_len = vl; }
      else        { d.u_off = a.u_len; d.u_len = vl; d.v_off = 0; d.v_len = ul; }
      const uint32_t top = a.limbs[d.u_off + d.u_len - 1];
      const uint32_t ubits = (d.u_len - 1) * 32u + (32u - __clz(top));
      uint32_t nq = 256;
      for (uint32_t k = 0; k < NA_MAX_NQ / 256; ++k)
        if (a.thr[k] != 0u && ubits >= a.thr[k]) nq += 256;
      d.nq = nq;
      d.out_off = 0;
      if (nq > NA_MAX_NQ) pre = MGCD_ERR_NOT_ENOUGH_MODULI;
    }
  }
  __syncthreads();
  if (pre != MGCD_OK) {
    if (threadIdx.x == 0) { *a.status = pre; *a.count = 0; }
    return;
  }
  uint32_t* u0 = a.scratch;
  uint32_t* v0 = a.scratch + NA_MAX_NQ;
  int2* hist = reinterpret_cast<int2*>(a.scratch + 2 * (size_t)NA_MAX_NQ);
  // caller-owned operand buffers carry no padding for widened bulk copies: plain loads
  const Stage stg{smem + 2 * NA_MAX_NQ, nullptr, nullptr, 0u};
  run_pair<NA_THREADS, SYNC_CTA>(a.limbs, d, a.mods, NA_L, 0u, d.nq, smem, smem + NA_MAX_NQ, stg,
                              rs, u0, v0, hist, nullptr, a.digits, a.count, &iters, a.status, InvTab{nullptr, 0u});
  if (threadIdx.x == 0) {
    const int32_t s = *a.status;
    *a.status = s == ST_OK ? MGCD_OK : (s == ST_REDUX || s == ST_INSUFFICIENT) ? MGCD_ERR_REDUX
              : s == ST_RECOVERY ? MGCD_ERR_RECOVERY : MGCD_ERR_KERNEL;
  }
}

std::mutex g_setup_mu;
unsigned long long g_ctx[NA_MAX_DEVICES];    // id of the CUDA context set up on each device (0: none)
uint32_t* g_scratch_addr[NA_MAX_DEVICES];
const ModConst* g_mods_addr[NA_MAX_DEVICES];
bool g_host_ready = false;
ModConstHost g_host_mods[NA_MAX_NQ];
uint32_t g_thr[NA_MAX_NQ / 256];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Unique id of the CUDA context that work on device dev runs in from this thread (0 on
// failure).  A device reset or a new context brings fresh, zeroed copies of the static
// arrays, so the set-up is cached per context id, not per device.  The driver functions
// come from the runtime's entry-point table (no link against the driver library).  A thread
// without a current context gets the device's primary context bound by cudaSetDevice, as
// the runtime would bind it for the launch.  Called with g_setup_mu held.
unsigned long long current_context_id(int dev)
{
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void* f1 = nullptr;
    void* f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return 0;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext c = nullptr;
  if (g_ctx_get_current(&c) != CUDA_SUCCESS) return 0;
  if (!c && (cudaSetDevice(dev) != cudaSuccess || g_ctx_get_current(&c) != CUDA_SUCCESS || !c)) return 0;
  unsigned long long id = 0;
  return g_ctx_get_id(c, &id) == CUDA_SUCCESS ? id : 0;
}

// Set-up of the current context on device dev: device addresses of the two arrays (host
// code may not use the arrays' names as addresses) and the moduli table copy.
int setup_device(int dev)
{
  std::lock_guard<std::mutex> lock(g_setup_mu);
  const unsigned long long ctx = current_context_id(dev);
  if (ctx == 0) return MGCD_ERR_NO_DEVICE;
  if (g_ctx[dev] == ctx) return MGCD_OK;
  if (!g_host_ready) {
    uint32_t q[NA_MAX_NQ];
    if (gen_moduli(NA_L, q, NA_MAX_NQ) != NA_MAX_NQ) return MGCD_ERR_KERNEL;
    mod_constants(q, NA_MAX_NQ, g_host_mods);
    // thresholds of the reference's moduli count (numModuliNeededFor), nondecreasing in bits
    uint32_t k = 0;
    std::memset(g_thr, 0, sizeof g_thr);
    for (uint32_t bits = 2; bits < 32u * NA_MAX_NQ && k < NA_MAX_NQ / 256; ++bits)
      while (k < NA_MAX_NQ / 256 && (uint32_t)moduli_needed(NA_L, bits) > 256u * (k + 1)) g_thr[k++] = bits;
    g_host_ready = true;
  }
  void* s = nullptr;
  void* m = nullptr;
  if (cudaGetSymbolAddress(&s, g_na_scratch) != cudaSuccess) return MGCD_ERR_CUDA;
  if (cudaGetSymbolAddress(&m, g_na_mods) != cudaSuccess) return MGCD_ERR_CUDA;
  if (cudaMemcpyToSymbol(g_na_mods, g_host_mods, sizeof(g_host_mods)) != cudaSuccess) return MGCD_ERR_CUDA;
  g_scratch_addr[dev] = static_cast<uint32_t*>(s);
  g_mods_addr[dev] = static_cast<const ModConst*>(m);
  g_ctx[dev] = ctx;
  return MGCD_OK;
}

}  // namespace
}  // namespace mgcd

using namespace mgcd;

extern "C" int mgcd_gcd_digits_noalloc(const uint32_t* d_limbs, size_t uSz, size_t vSz, mgcd_pair* d_digits,
                                       size_t cap, uint32_t* d_count, int32_t* d_status, void* stream)
{
  if (!d_limbs || !d_digits || !d_count || !d_status || uSz == 0 || vSz == 0) return MGCD_ERR_INVALID_ARG;
  if (uSz > 32u * NA_MAX_NQ || vSz > 32u * NA_MAX_NQ) return MGCD_ERR_NOT_ENOUGH_MODULI;
  const size_t bound_bits = 32 * (uSz > vSz ? uSz : vSz);
  const int bound_nq = moduli_needed(NA_L, bound_bits);
  if (bound_nq > (int)NA_MAX_NQ) return MGCD_ERR_NOT_ENOUGH_MODULI;
  if (cap < (size_t)bound_nq) return MGCD_ERR_CAPACITY;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MGCD_ERR_NO_DEVICE;
  if (dev < 0 || dev >= NA_MAX_DEVICES) return MGCD_ERR_NO_DEVICE;
  const int rc = setup_device(dev);
  if (rc != MGCD_OK) return rc;

  NaArgs a;
  a.limbs = d_limbs;
  a.u_len = (uint32_t)uSz;
  a.v_len = (uint32_t)vSz;
  a.scratch = g_scratch_addr[dev];
  a.mods = g_mods_addr[dev];
  std::memcpy(a.thr, g_thr, sizeof a.thr);
  a.digits = d_digits;
  a.count = d_count;
  a.status = d_status;
  const size_t smem = sizeof(uint32_t) * (2 * (size_t)NA_MAX_NQ + CHUNK);
  // the launch's own return code: an error left pending by earlier, unrelated calls is
  // neither blamed on this call nor cleared
  void* args[] = {&a};
  const cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(&noalloc_kernel), dim3(1), dim3(NA_THREADS),
                                         args, smem, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? MGCD_OK : MGCD_ERR_CUDA;
}
