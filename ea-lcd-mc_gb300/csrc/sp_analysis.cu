// sp_analysis.cu -- configuration analysis of sample-packed jobs: plane
// overlaps of replica pairs and their correlation functions along the tube.
//
// The reference ships no analysis code; its data description (DATA/README.md)
// names the ingredients: correlation functions built from basis functions
// f, g in {x, x^3, sign x} of the overlap, computed with r = 2, 4, 6, 8
// replicas, and the 3 x 3 (and 2 x 2) matrices of those correlations per
// distance.  The definition used here:
//
//   plane overlap   q_z = (1/L^2) sum over the plane z of s^a s^c, for the
//                   replica pairs (a, c) = (0,1), (2,3), ... among the first
//                   r replicas, at each temperature slot (the configuration
//                   the slot holds);
//   correlation     C_fg(d) = < f(q_z) g(q_{z+d}) >, averaged over the pairs
//                   and the planes z (z + d taken modulo Lz under PBC; only
//                   z + d < Lz under open boundaries).
//
// Two kernels: bit-sliced counts of the differing spins of each (word, pair,
// slot, plane) for the 64 samples of a word, then one thread per (sample,
// slot, distance) summing the nine products in a fixed order (FP64).
#include <cstdint>

#include "kernels_dev.cuh"
#include "sp.cuh"

namespace eagb {

void set_last_error(const char *msg);  // api.cu

constexpr int kPlanePlanes = 12;  // bit planes of a plane's count: L^2 < 4096

// diff[w][sample][pair][slot][z] = spins that differ between the pair's two
// replicas on plane z.  One thread per (word, pair, slot, plane).
__global__ void __launch_bounds__(128) k_sp_plane_diff(const __grid_constant__ SpDev d, int npairs, int32_t *diff) {
  const int NB = d.NB, NR = d.NR, G = NR * NB, Lz = d.Lz, L2 = d.L * d.L;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.nw * npairs * NB * Lz) return;
  const int z = (int)(t % Lz), b = (int)((t / Lz) % NB), k = (int)((t / ((long long)Lz * NB)) % npairs);
  const int w = (int)(t / ((long long)Lz * NB * npairs));
  const u64 *Sa = d.S + ((size_t)w * d.V + (size_t)z * L2) * G + (size_t)(2 * k) * NB + b;
  u64 P[kPlanePlanes];
#pragma unroll
  for (int q = 0; q < kPlanePlanes; ++q) P[q] = 0;
  for (int i = 0; i < L2; ++i) {
    u64 c = __ldg(Sa + (size_t)i * G) ^ __ldg(Sa + (size_t)i * G + NB);
#pragma unroll
    for (int q = 0; q < kPlanePlanes; ++q) {
      const u64 h = P[q] & c;
      P[q] ^= c;
      c = h;
    }
  }
  int32_t *o = diff + ((((size_t)w * 64) * npairs + k) * NB + b) * Lz + z;
  const size_t lane_stride = (size_t)npairs * NB * Lz;
  for (int lane = 0; lane < 64; ++lane) {
    int n = 0;
#pragma unroll
    for (int q = 0; q < kPlanePlanes; ++q) n |= (int)((P[q] >> lane) & 1ull) << q;
    o[lane * lane_stride] = n;
  }
}

__device__ __forceinline__ void basis3(double x, double f[3]) {
  f[0] = x;
  f[1] = __dmul_rn(__dmul_rn(x, x), x);
  f[2] = x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0);
}

// C[w*64 + sample][slot][d][3][3] = the correlation matrix at distance d
// (sums over pairs and planes in a fixed order, then divided by their count).
__global__ void __launch_bounds__(128) k_sp_plane_corr(const __grid_constant__ SpDev d, int npairs, int dmax,
                                                       const int32_t *diff, double *C) {
  const int NB = d.NB, Lz = d.Lz, L2 = d.L * d.L;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.nw * 64 * NB * (dmax + 1)) return;
  const int dd = (int)(t % (dmax + 1)), b = (int)((t / (dmax + 1)) % NB);
  const long long smp = t / ((long long)(dmax + 1) * NB);  // w * 64 + sample
  const bool pbc = d.bc == EA_PBC;
  double acc[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[q] = 0.0;
  const double inv = 1.0 / (double)L2;
  long long n = 0;
  for (int k = 0; k < npairs; ++k) {
    const int32_t *row = diff + (((size_t)smp * npairs + k) * NB + b) * Lz;
    const int zmax = pbc ? Lz : Lz - dd;
    for (int z = 0; z < zmax; ++z) {
      const int z2 = pbc ? (z + dd) % Lz : z + dd;
      const double x1 = __dsub_rn(1.0, __dmul_rn(2.0 * inv, (double)row[z]));
      const double x2 = __dsub_rn(1.0, __dmul_rn(2.0 * inv, (double)row[z2]));
      double f[3], g[3];
      basis3(x1, f);
      basis3(x2, g);
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) acc[p * 3 + q] = __dadd_rn(acc[p * 3 + q], __dmul_rn(f[p], g[q]));
      ++n;
    }
  }
  double *o = C + (size_t)t * 9;
  for (int q = 0; q < 9; ++q) o[q] = n ? acc[q] / (double)n : 0.0;
}

}  // namespace eagb

using namespace eagb;

extern "C" {

// Defined in sp.cu: the job's device view and stream.
int ea_sp_device_view(ea_sp *job, SpDev *d, cudaStream_t *st);

static int an_fail(const char *m) {
  set_last_error(m);
  return EA_ERR_ARG;
}

int ea_sp_plane_overlaps(ea_sp *job, int32_t nrep, int32_t *diff) {
  SpDev d;
  cudaStream_t st;
  int rc = ea_sp_device_view(job, &d, &st);
  if (rc) return rc;
  if (!diff || nrep < 2 || (nrep & 1) || nrep > d.NR) return an_fail("nrep: an even number of replicas, 2..NR");
  if (d.L * d.L >= (1 << kPlanePlanes)) return an_fail("planes of at most 4095 sites");
  const int npairs = nrep / 2;
  const size_t n = (size_t)d.nw * 64 * npairs * d.NB * d.Lz;
  int32_t *dd = nullptr;
  cudaError_t e = cudaMalloc((void **)&dd, n * 4);
  const long long nt = (long long)d.nw * npairs * d.NB * d.Lz;
  if (e == cudaSuccess) {
    k_sp_plane_diff<<<(unsigned)((nt + 127) / 128), 128, 0, st>>>(d, npairs, dd);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(diff, dd, n * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (dd) cudaFree(dd);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return EA_ERR_CUDA;
  }
  return EA_OK;
}

int ea_sp_plane_correlations(ea_sp *job, int32_t nrep, int32_t dmax, double *C) {
  SpDev d;
  cudaStream_t st;
  int rc = ea_sp_device_view(job, &d, &st);
  if (rc) return rc;
  if (!C || nrep < 2 || (nrep & 1) || nrep > d.NR) return an_fail("nrep: an even number of replicas, 2..NR");
  if (dmax < 0 || dmax >= d.Lz) return an_fail("dmax: 0..Lz-1");
  if (d.L * d.L >= (1 << kPlanePlanes)) return an_fail("planes of at most 4095 sites");
  const int npairs = nrep / 2;
  const size_t nd = (size_t)d.nw * 64 * npairs * d.NB * d.Lz, nc = (size_t)d.nw * 64 * d.NB * (dmax + 1) * 9;
  int32_t *dd = nullptr;
  double *dc = nullptr;
  cudaError_t e = cudaMalloc((void **)&dd, nd * 4);
  if (e == cudaSuccess) e = cudaMalloc((void **)&dc, nc * 8);
  if (e == cudaSuccess) {
    const long long nt = (long long)d.nw * npairs * d.NB * d.Lz;
    k_sp_plane_diff<<<(unsigned)((nt + 127) / 128), 128, 0, st>>>(d, npairs, dd);
    const long long nt2 = (long long)d.nw * 64 * d.NB * (dmax + 1);
    k_sp_plane_corr<<<(unsigned)((nt2 + 127) / 128), 128, 0, st>>>(d, npairs, dmax, dd, dc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(C, dc, nc * 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (dd) cudaFree(dd);
  if (dc) cudaFree(dc);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return EA_ERR_CUDA;
  }
  return EA_OK;
}

}  // extern "C"
