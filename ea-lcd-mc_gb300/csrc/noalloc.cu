// noalloc.cu -- energy measurement that allocates no device memory.
//
// Some callers cannot call cudaMalloc: host frameworks that own every device
// byte through their own pool (an allocation behind their back breaks their
// accounting, and fails outright when the pool already holds the memory), and
// latency-critical loops that must not take the device-wide synchronisation
// an allocation may imply.  ea_measure_energy_noalloc serves them: it
// computes the same energies as ea_measure_energy for spins and couplings that
// the caller already keeps in device memory, and writes them to a caller
// buffer.  Its scratch space -- the per-tile partial sums of the energy kernel
// and the neighbour tables of the geometry -- is the file-scope array below,
// which every GPU that loads libeagb.so holds until the process exits.
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "eagb.h"
#include "host.hpp"
#include "kernels.cuh"

namespace eagb {
namespace {

// Scratch limits: at most kMaxPartials per-tile energy sums and kMaxHalf
// half-sites per parity (e.g. L = 32, Lz = 256).
constexpr size_t kMaxPartials = (size_t)1 << 20;  // 4 MiB of int32
constexpr int kMaxHalf = 8192;
constexpr size_t kPartBytes = kMaxPartials * 4;
constexpr size_t kIdxBytes = (size_t)12 * kMaxHalf * 4;
constexpr size_t kFlagBytes = (size_t)2 * kMaxHalf;
constexpr size_t kScratchBytes = kPartBytes + kIdxBytes + kFlagBytes;  // 4.4 MiB

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Device address of g_scratch per device, with the context it was looked up
// in: a recreated context (cudaDeviceReset) reloads the module, and the
// array may then sit at another address.
void *g_addr[kMaxDevices] = {};
CUcontext g_ctx[kMaxDevices] = {};

// The calling thread's current context (driver entry point looked up at run
// time; the library does not link the driver library).  nullptr if the
// lookup fails, which keeps one address per device.
CUcontext current_context() {
  using GetCurrent = CUresult (*)(CUcontext *);
  static GetCurrent fn = []() -> GetCurrent {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, CUDA_VERSION, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<GetCurrent>(f);
  }();
  CUcontext c = nullptr;
  if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

// Neighbour half indices and flags of the multispin lattice, written into the
// scratch tables (same tables as the context builds on the host: wrap-around
// rotation bits 0-5, top plane bit 6, bottom plane bit 7).
__global__ void k_noalloc_tables(int msc_l, int msc_lz, int half) {
  int32_t *idx = reinterpret_cast<int32_t *>(g_scratch + kPartBytes);
  uint8_t *flags = g_scratch + kPartBytes + kIdxBytes;
  const int msc_s = msc_l * msc_l, msc_v = msc_s * msc_lz;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= msc_v) return;
  const int side[3] = {msc_l, msc_l, msc_lz}, off[3] = {1, msc_l, msc_s};
  const int x[3] = {m % msc_l, (m / msc_l) % msc_l, m / msc_s};
  const int p = (x[0] + x[1] + x[2]) & 1, k = m >> 1;
  uint8_t f = 0;
  for (int d = 0; d < 6; ++d) {
    const int dim = d % 3, step = d < 3 ? 1 : -1;
    int y[3] = {x[0], x[1], x[2]};
    y[dim] = (x[dim] + step + side[dim]) % side[dim];
    const int mn = y[0] + y[1] * msc_l + y[2] * msc_s;
    idx[(p * 6 + d) * half + k] = mn >> 1;
    if (mn - m != step * off[dim]) f |= (uint8_t)(1u << d);
  }
  if (x[2] == msc_lz - 1) f |= 0x40;
  if (x[2] == 0) f |= 0x80;
  flags[p * half + k] = f;
}

}  // namespace

void set_last_error(const char *msg);
}  // namespace eagb

using namespace eagb;

extern "C" int ea_measure_energy_noalloc(const ea_geom *gp, const uint64_t *d_spins, const uint64_t *d_couplings,
                                         int32_t *d_energies, void *stream) {
  Geometry g;
  if (!gp || !g.set(*gp) || !d_spins || !d_couplings || !d_energies) {
    set_last_error("ea_measure_energy_noalloc: bad geometry or null pointer");
    return EA_ERR_ARG;
  }
  if (g.NR != 8 && g.NR != 4 && g.NR != 2) {
    set_last_error("ea_measure_energy_noalloc: NR must be 2, 4 or 8");
    return EA_ERR_ARG;
  }
  const int kt = g.NR == 8 ? 4 : g.NR == 4 ? 8 : 16;
  const int ntiles = (g.half + kt - 1) / kt;
  if (g.half > kMaxHalf || (size_t)ntiles * g.ns * g.NB * g.NR > kMaxPartials) {
    set_last_error("ea_measure_energy_noalloc: job exceeds the fixed scratch (needs (L/4)^2 (Lz/4)/2 <= 8192 "
                   "and ceil(half/KT) * nsamples * NB * NR <= 1048576, KT = 32/NR)");
    return EA_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_last_error("ea_measure_energy_noalloc: no current CUDA device");
    return EA_ERR_CUDA;
  }
  // an error left by the caller's own earlier work is theirs: report it and
  // leave it pending instead of taking it for a failure of the launches below
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess) {
    char msg[256];
    std::snprintf(msg, sizeof(msg), "ea_measure_energy_noalloc: a CUDA error is pending from earlier work: %s",
                  cudaGetErrorString(pending));
    set_last_error(msg);
    return EA_ERR_CUDA;
  }
  unsigned char *base;
  {
    // once per device (and again if its context was recreated), with that
    // device current: the device address of the scratch array (the host-side
    // name g_scratch is not a device address)
    std::lock_guard<std::mutex> lock(g_mu);
    const CUcontext ctx = current_context();
    if (!g_addr[dev] || g_ctx[dev] != ctx) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) {
        set_last_error("ea_measure_energy_noalloc: cudaGetSymbolAddress of the scratch array failed");
        return EA_ERR_CUDA;
      }
      g_addr[dev] = p;
      g_ctx[dev] = ctx;
    }
    base = static_cast<unsigned char *>(g_addr[dev]);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  JobDev j{};
  j.NB = g.NB; j.NR = g.NR; j.ns = g.ns; j.half = g.half; j.msc_l = g.msc_l; j.msc_s = g.msc_s;
  j.msc_lz = g.msc_lz; j.L = g.L; j.Lz = g.Lz; j.V = g.V; j.bc = g.bc;
  j.kt = kt; j.ntiles = ntiles;
  set_dividers(j);
  j.spins = const_cast<unsigned long long *>(reinterpret_cast<const unsigned long long *>(d_spins));
  j.J = reinterpret_cast<const unsigned long long *>(d_couplings);
  j.epart = reinterpret_cast<int32_t *>(base);
  j.nbidx = reinterpret_cast<const int32_t *>(base + kPartBytes);
  j.nbflag = base + kPartBytes + kIdxBytes;
  j.E = d_energies;
  // each launch checked right after it is made
  const char *failed = nullptr;
  cudaError_t e;
  k_noalloc_tables<<<(g.msc_v + 255) / 256, 256, 0, st>>>(g.msc_l, g.msc_lz, g.half);
  if ((e = cudaGetLastError()) != cudaSuccess) failed = "neighbour tables";
  else if ((e = launch_energy(j, st)) != cudaSuccess) failed = "energy partial sums";
  else if ((e = launch_energy_reduce(j, st)) != cudaSuccess) failed = "energy reduction";
  if (failed) {
    char msg[256];
    std::snprintf(msg, sizeof(msg), "ea_measure_energy_noalloc: launch of the %s kernel failed: %s", failed,
                  cudaGetErrorString(e));
    set_last_error(msg);
    return EA_ERR_CUDA;
  }
  return EA_OK;
}
