// GmpCudaDevice.cpp -- the drop-in GmpCuda::GmpCudaDevice (include/GmpCuda.h) over the C ABI.
//
// Mirrors the reference's host object (GmpCudaDevice.cu:96-144, GmpCudaDevice-gcd.cu:57-132):
// one context per object (moduli table uploaded once), gcd() blocking on the device.
#include "GmpCuda.h"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "modgcd.h"

using namespace GmpCuda;

namespace {

[[noreturn]] void fail(int rc)
{
  throw std::runtime_error(mgcd_status_string(rc));
}

// |x| as little-endian 32-bit limbs (mpz_export(buf, &n, -1, 4, 0, 0, x), GmpCudaDevice-gcd.cu:72).
void export_limbs(mpz_srcptr x, std::vector<uint32_t>& out)
{
  out.resize((mpz_sizeinbase(x, 2) + 31) / 32 + 1);
  size_t n = 0;
  if (mpz_sgn(x) != 0) mpz_export(out.data(), &n, -1, sizeof(uint32_t), 0, 0, x);
  out.resize(n);
}

}  // namespace

void GmpCudaDevice::setDevice(int devNo)
{
  const int rc = mgcd_set_device(devNo);
  if (rc == MGCD_ERR_NO_DEVICE) throw std::runtime_error("Invalid device number.");
  if (rc != MGCD_OK) fail(rc);
}

GmpCudaDevice::GmpCudaDevice(void) : ctx(nullptr), deviceNum(-1), maxGridSize(0)
{
  const int rc = mgcd_create(-1, L, &ctx);
  if (rc != MGCD_OK) fail(rc);
  mgcd_max_grid_size(ctx, &maxGridSize);
}

GmpCudaDevice::~GmpCudaDevice()
{
  if (ctx) mgcd_destroy(ctx);
}

void GmpCudaDevice::gcd(mpz_t g, mpz_t u, mpz_t v)
{
  if (mpz_cmp(u, v) < 0) mpz_swap(u, v);
  static thread_local std::vector<uint32_t> ul, vl, gl;
  export_limbs(u, ul);
  export_limbs(v, vl);
  gl.resize(std::max(ul.size(), vl.size()) + 1);
  size_t glen = 0;
  const int rc = mgcd_gcd(ctx, ul.data(), ul.size(), vl.data(), vl.size(), gl.data(), gl.size(), &glen);
  if (rc != MGCD_OK) fail(rc);
  mpz_import(g, glen, -1, sizeof(uint32_t), 0, 0, gl.data());
}

void GmpCudaDevice::gcdBatch(size_t n, mpz_ptr g, mpz_srcptr u, mpz_srcptr v)
{
  if (n == 0) return;
  std::vector<uint32_t> limbs, x;
  std::vector<uint64_t> uo(n), vo(n), go(n);
  std::vector<uint32_t> un(n), vn(n), gc(n), gn(n);
  std::vector<int32_t> st(n);
  uint64_t gtot = 0;
  for (size_t i = 0; i < n; ++i) {
    export_limbs(&u[i], x);
    uo[i] = limbs.size();
    un[i] = (uint32_t)x.size();
    limbs.insert(limbs.end(), x.begin(), x.end());
    export_limbs(&v[i], x);
    vo[i] = limbs.size();
    vn[i] = (uint32_t)x.size();
    limbs.insert(limbs.end(), x.begin(), x.end());
    go[i] = gtot;
    gc[i] = std::max(un[i], vn[i]) + 1;
    gtot += gc[i];
  }
  std::vector<uint32_t> gbuf(gtot);
  const int rc = mgcd_gcd_batch(ctx, n, limbs.data(), uo.data(), un.data(), vo.data(), vn.data(), gbuf.data(),
                                go.data(), gc.data(), gn.data(), st.data());
  if (rc != MGCD_OK) fail(rc);
  for (size_t i = 0; i < n; ++i) mpz_import(&g[i], gn[i], -1, sizeof(uint32_t), 0, 0, gbuf.data() + go[i]);
}
