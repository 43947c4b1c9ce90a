/*  GmpCuda.h -- drop-in C++ API of the GB300 modular integer GCD (libGmpCuda.so).

    Same namespace, class, method and constant names as the reference's GmpCuda.h
    (mountunion/ModGCD-OneGPU GmpCuda.h:22-127), so code written against the reference
    (its testmodgcd.cpp, for one) compiles and links unchanged against this header plus
    -lGmpCuda -lmodgcd -l:libgmp.so.10.  Host compilers only: nothing here needs nvcc.

    Behaviour kept from the reference:
      - gcd(g, u, v) swaps u and v in place when u < v (GmpCudaDevice-gcd.cu:61-62) and
        returns |gcd| in g (:129);
      - errors are std::runtime_error with the reference's messages (:78, :82, :107-109)
        and "Invalid device number." from setDevice (GmpCudaDevice.cu:100-101);
      - moduli[] is the createModuli table (descending L-bit primes passing the
        Cavagnino-Werbrouck test), generated at build time in the reference's format.
    Differences: zero operands follow mpz_gcd (gcd(x, 0) = |x|) instead of the reference
    kernel's undefined result; the table holds NUM_MODULI = 131,072 moduli (the reference:
    65,536), so operands up to ~1.6 Mbit are accepted; the object is not copyable.
    Added: gcdBatch (many pairs in one persistent launch).
*/
#ifndef GMPCUDA_DROPIN_H
#define GMPCUDA_DROPIN_H

#include <gmp.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>

struct mgcd_context;

namespace GmpCuda
{
  constexpr int WARP_SZ = 32;

  class GmpCudaDevice
  {
  private:
    mgcd_context* ctx;
    int deviceNum;
    int maxGridSize;
  public:
    static constexpr int GCD_BLOCK_SZ = WARP_SZ << 3;
    static constexpr int MAX_THREADS  = GCD_BLOCK_SZ * GCD_BLOCK_SZ;
    static constexpr uint32_t GCD_KERNEL_ERROR   = 0;
    static constexpr uint32_t GCD_REDUX_ERROR    = 0;
    static constexpr uint32_t GCD_RECOVERY_ERROR = 1;
    typedef struct alignas(8) {uint32_t modulus; int32_t value;} pair_t;

    static void setDevice(int devNo = 0);
    GmpCudaDevice(void);
    ~GmpCudaDevice();
    GmpCudaDevice(const GmpCudaDevice&) = delete;
    GmpCudaDevice& operator=(const GmpCudaDevice&) = delete;

    void gcd(mpz_t g, mpz_t u, mpz_t v);  // throw (std::runtime_error)
    int getMaxGridSize(void) const {return maxGridSize;}

    //  g[i] = gcd(u[i], v[i]) for i < n, all pairs in one batched launch.  Operands are
    //  not modified.  Throws std::runtime_error on the first failing pair.
    void gcdBatch(size_t n, mpz_ptr g, mpz_srcptr u, mpz_srcptr v);
  };

  constexpr int L          = 32;
  constexpr int W          = 64;
  constexpr int NUM_MODULI = 131072;

  extern const uint32_t moduli[];
  //  Multiply-by-inverse constants J = floor(2^(W+L-1) / moduli[i]) + 1 of the reference's
  //  mod() (GmpCudaDevice-getGcdKernel.cu:248-251, 332-340), tabulated instead of recomputed.
  extern const uint64_t moduliInverse[];
}

#endif
