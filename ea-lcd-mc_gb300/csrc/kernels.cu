// kernels.cu -- the one-job kernels of the EA-LCD-MC hot path (bodies in
// kernels_dev.cuh) and their launchers.
#include "kernels_dev.cuh"

#include <cstdio>

namespace eagb {

bool slab_shape(const JobDev &j, int *D, int *P, int *nslab) {
  const int S = j.L * j.L;
  if (S > 1024) return false;
  const int d = j.Lz < kSlabSites / S ? j.Lz : kSlabSites / S;
  int p = 512 / S;
  if (p > d) p = d;
  if (p < 1) p = 1;
  if ((d + p - 1) / p > kSlabMaxPerThread) return false;
  *D = d; *P = p; *nslab = (j.Lz + d - 1) / d;
  return true;
}

void set_dividers(JobDev &j) {
  j.fd_L.set(j.L); j.fd_S.set(j.L * j.L); j.fd_ml.set(j.msc_l); j.fd_mlz.set(j.msc_lz);
  j.fd_hl.set(j.msc_l / 2); j.fd_nclust.set(j.nclust > 0 ? j.nclust : 1);
}

__global__ void k_fill_bits(const __grid_constant__ JobDev j, int parity) { fill_bits_body(j, parity); }

template <int NR, int KT, bool UPDATE>
__global__ void __launch_bounds__(512, 2) k_sweep(const __grid_constant__ JobDev j, int parity, int energy) {
  extern __shared__ __align__(16) unsigned char smem[];
  sweep_body<NR, KT, UPDATE>(j, blockIdx.x, parity, energy, smem);
}

__global__ void k_energy_reduce(const __grid_constant__ JobDev j) {
  energy_reduce_body(j, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(256) k_pt(const __grid_constant__ JobDev j) {
  __shared__ u64 s_ira[8][256];
  __shared__ uint8_t s_wc[8][256];
  pt_body(j, blockIdx.x, blockIdx.y, s_ira, s_wc);
}

__global__ void k_measure(const __grid_constant__ JobDev j, int itm) {
  measure_body(j, blockIdx.x * blockDim.x + threadIdx.x, itm);
}

__global__ void k_hou_pairs(const __grid_constant__ JobDev j) { pairs_body(j); }

__global__ void k_hou_overlap(const __grid_constant__ JobDev j, int g) {
  overlap_body(j, g, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

__global__ void __launch_bounds__(1024, 2) k_cc_slab(const __grid_constant__ JobDev j, int D, int P) {
  __shared__ uint32_t lab[kSlabSites];
  __shared__ uint8_t qs[kSlabSites];
  cc_slab_body(j, D, P, blockIdx.x, blockIdx.y, lab, qs);
}

__global__ void k_cc_merge(const __grid_constant__ JobDev j, int D, int nslab) {
  cc_merge_body(j, D, nslab, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

__global__ void k_cc_compress(const __grid_constant__ JobDev j, int D, int nslab) {
  cc_compress_body(j, D, nslab, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

__global__ void __launch_bounds__(512) k_hou_flip(const __grid_constant__ JobDev j, int g) {
  extern __shared__ uint32_t s_flip[];
  flip_body(j, j.U, g, blockIdx.x, s_flip + 64, reinterpret_cast<int *>(s_flip));
}

size_t flip_smem_bytes(const JobDev &j) { return 256 + (size_t)j.V / 8; }

__global__ void __launch_bounds__(256) k_hou_select(const __grid_constant__ JobDev j) {
  select_body(j, j.U, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

__global__ void __launch_bounds__(256) k_hou_apply(const __grid_constant__ JobDev j, int g) {
  __shared__ unsigned s_sel[8];
  apply_body(j, g, blockIdx.x, blockIdx.y, s_sel);
}

// Bonds between equal-overlap neighbours towards -x, -y (periodic) and -z
// (periodic under PBC, none across z = 0 under OBC); the initial label is the
// smallest bonded index (HoudayerXEA.cu:77-121).
__global__ void k_cc_init(JobDev j) {
  const size_t n = (size_t)j.ns * j.nclust * j.V;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const size_t lat = t / j.V;
  const int i = (int)(t % j.V), L = j.L, S = L * L;
  const int x = i % L, y = (i / L) % L, z = i / S;
  const u64 *Q = j.Q + lat * 2 * j.half;
  const int q = q_bit(j, Q, x, y, z);
  uint32_t m = (uint32_t)i;
  const int xm = x == 0 ? L - 1 : x - 1, ym = y == 0 ? L - 1 : y - 1;
  if (q_bit(j, Q, xm, y, z) == q) m = min(m, (uint32_t)(xm + L * y + S * z));
  if (q_bit(j, Q, x, ym, z) == q) m = min(m, (uint32_t)(x + L * ym + S * z));
  if (z > 0 || j.bc == EA_PBC) {
    const int zm = z == 0 ? j.Lz - 1 : z - 1;
    if (q_bit(j, Q, x, y, zm) == q) m = min(m, (uint32_t)(x + L * y + S * zm));
  }
  j.label[t] = m;
}

// Planes of 1025..8192 sites: a CTA-wide loop over the slab's sites.
__global__ void __launch_bounds__(512) k_cc_local(JobDev j, int D) {
  __shared__ uint32_t lab[kSlabSites];
  __shared__ uint8_t qs[kSlabSites];
  const int L = j.L, S = L * L, tid = threadIdx.x, nth = blockDim.x;
  const size_t lat = blockIdx.y;
  const int z0 = blockIdx.x * D, nz = min(D, j.Lz - z0), n = S * nz;
  const u64 *Q = j.Q + lat * 2 * j.half;
  for (int i = tid; i < n; i += nth) {
    const int zl = j.fd_S.div(i), xy = i - zl * S, y = j.fd_L.div(xy), x = xy - y * L;
    qs[i] = (uint8_t)q_bit(j, Q, x, y, z0 + zl);
    lab[i] = (uint32_t)i;
  }
  __syncthreads();
  for (int i = tid; i < n; i += nth) {
    const int zl = j.fd_S.div(i), xy = i - zl * S, y = j.fd_L.div(xy), x = xy - y * L, q = qs[i];
    const int xm = x == 0 ? L - 1 : x - 1, ym = y == 0 ? L - 1 : y - 1;
    // site 0 tests its x-wrap bond against x = cc_xq (see JobDev::cc_xq)
    const int xt = (z0 == 0 && i == 0) ? j.cc_xq : xm;
    if (qs[xt + L * y + S * zl] == q) cc_unite(lab, (uint32_t)i, (uint32_t)(xm + L * y + S * zl));
    if (qs[x + L * ym + S * zl] == q) cc_unite(lab, (uint32_t)i, (uint32_t)(x + L * ym + S * zl));
    if (zl > 0 && qs[i - S] == q) cc_unite(lab, (uint32_t)i, (uint32_t)(i - S));
  }
  __syncthreads();
  uint32_t *glab = j.label + lat * j.V + (size_t)z0 * S;
  const uint32_t off = (uint32_t)z0 * S;
  for (int i = tid; i < n; i += nth) glab[i] = off + cc_find(lab, (uint32_t)i);
}

// Label reduction of Komura (HoudayerXEA.cu:254-331): every bond that is not
// the initial tree edge is merged with atomicMin, so each root ends as the
// smallest site index of its cluster.
__global__ void k_cc_union(JobDev j) {
  const size_t n = (size_t)j.ns * j.nclust * j.V;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const size_t lat = t / j.V;
  const int i = (int)(t % j.V), L = j.L, S = L * L;
  const int x = i % L, y = (i / L) % L, z = i / S;
  const u64 *Q = j.Q + lat * 2 * j.half;
  uint32_t *lab = j.label + lat * j.V;
  const int q = q_bit(j, Q, x, y, z);
  const int xm = x == 0 ? L - 1 : x - 1, ym = y == 0 ? L - 1 : y - 1;
  // site 0 tests its x-wrap bond against x = cc_xq (see JobDev::cc_xq)
  const int xt = i == 0 ? j.cc_xq : xm;
  if (q_bit(j, Q, xt, y, z) == q) cc_unite(lab, (uint32_t)i, (uint32_t)(xm + L * y + S * z));
  if (q_bit(j, Q, x, ym, z) == q) cc_unite(lab, (uint32_t)i, (uint32_t)(x + L * ym + S * z));
  if (z == 0 && j.bc == EA_PBC && q_bit(j, Q, x, y, j.Lz - 1) == q)
    cc_unite(lab, (uint32_t)i, (uint32_t)(x + L * y + S * (j.Lz - 1)));
}

__global__ void k_cc_flatten(JobDev j) {
  const size_t n = (size_t)j.ns * j.nclust * j.V;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const size_t lat = t / j.V;
  uint32_t *lab = j.label + lat * j.V;
  j.label[t] = cc_find(lab, (uint32_t)(t % j.V));
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
int sweep_kt(const JobDev &j) { return j.kt; }

size_t sweep_smem_bytes(const JobDev &j) { return sweep_smem_for(j.NB, j.NR, j.kt); }

template <int NR, int KT>
static cudaError_t launch_sweep_t(const JobDev &j, int parity, bool energy, bool update, cudaStream_t st) {
  if (update) {
    const size_t sm = sweep_smem_bytes(j);
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_sweep<NR, KT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      attr = true;
    }
    k_sweep<NR, KT, true><<<j.ntiles, 512, sm, st>>>(j, parity, energy ? 1 : 0);
  } else {
    k_sweep<NR, KT, false><<<j.ntiles, 512, (size_t)KT * 8 * 4, st>>>(j, parity, 1);
  }
  return cudaGetLastError();
}

static cudaError_t dispatch_sweep(const JobDev &j, int parity, bool energy, bool update, cudaStream_t st) {
  switch (j.NR * 100 + j.kt) {
    case 801: return launch_sweep_t<8, 1>(j, parity, energy, update, st);
    case 802: return launch_sweep_t<8, 2>(j, parity, energy, update, st);
    case 804: return launch_sweep_t<8, 4>(j, parity, energy, update, st);
    case 402: return launch_sweep_t<4, 2>(j, parity, energy, update, st);
    case 404: return launch_sweep_t<4, 4>(j, parity, energy, update, st);
    case 408: return launch_sweep_t<4, 8>(j, parity, energy, update, st);
    case 204: return launch_sweep_t<2, 4>(j, parity, energy, update, st);
    case 208: return launch_sweep_t<2, 8>(j, parity, energy, update, st);
    case 216: return launch_sweep_t<2, 16>(j, parity, energy, update, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_fill_bits(const JobDev &j, int parity, cudaStream_t st) {
  k_fill_bits<<<1, 64, 0, st>>>(j, parity);
  return cudaGetLastError();
}

cudaError_t launch_sweep(const JobDev &j, int parity, bool energy, cudaStream_t st) {
  return dispatch_sweep(j, parity, energy, true, st);
}

cudaError_t launch_energy(const JobDev &j, cudaStream_t st) {
  return dispatch_sweep(j, 0, true, false, st);
}

cudaError_t launch_energy_reduce(const JobDev &j, cudaStream_t st) {
  const int n = j.ns * j.NB * j.NR;
  k_energy_reduce<<<(n + 255) / 256, 256, 0, st>>>(j);
  return cudaGetLastError();
}

cudaError_t launch_pt(const JobDev &j, cudaStream_t st) {
  dim3 grid(j.ns, (j.NR + 7) / 8);
  k_pt<<<grid, 256, 0, st>>>(j);
  return cudaGetLastError();
}

cudaError_t launch_measure(const JobDev &j, int itm, cudaStream_t st) {
  const int n = j.ns * j.NB * j.NR;
  k_measure<<<(n + 255) / 256, 256, 0, st>>>(j, itm);
  return cudaGetLastError();
}

cudaError_t launch_houdayer_pairs(const JobDev &j, cudaStream_t st) {
  k_hou_pairs<<<1, 1, 0, st>>>(j);
  return cudaGetLastError();
}

cudaError_t launch_houdayer_group(const JobDev &j, int g, cudaStream_t st) {
  const size_t ns = (size_t)j.ns * j.nclust * j.V;
  const unsigned bs = (unsigned)((ns + 255) / 256);
  const unsigned nlat = (unsigned)(j.ns * j.nclust);
  k_hou_overlap<<<dim3((2 * j.half + 255) / 256, nlat), 256, 0, st>>>(j, g);
  int D, P, nslab;
  if (slab_shape(j, &D, &P, &nslab)) {
    k_cc_slab<<<dim3(nslab, nlat), j.L * j.L * P, 0, st>>>(j, D, P);
    k_cc_merge<<<dim3((nslab * j.L * j.L + 255) / 256, nlat), 256, 0, st>>>(j, D, nslab);
    k_cc_compress<<<dim3((nslab * j.L * j.L + 255) / 256, nlat), 256, 0, st>>>(j, D, nslab);
    const size_t sm = flip_smem_bytes(j);
    if (sm <= kFlipMaxSmem) {
      static bool attr = false;
      if (!attr) {
        cudaFuncSetAttribute(k_hou_flip, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFlipMaxSmem);
        attr = true;
      }
      k_hou_flip<<<nlat, 512, sm, st>>>(j, g);
      return cudaGetLastError();
    }
  } else {
    const int S = j.L * j.L;
    if (S <= kSlabSites) {
      D = min(j.Lz, kSlabSites / S);
      nslab = (j.Lz + D - 1) / D;
      k_cc_local<<<dim3(nslab, nlat), 512, 0, st>>>(j, D);
      k_cc_merge<<<dim3((nslab * S + 255) / 256, nlat), 256, 0, st>>>(j, D, nslab);
    } else {
      // planes too large for SMEM: Komura's passes on global labels
      k_cc_init<<<bs, 256, 0, st>>>(j);
      k_cc_flatten<<<bs, 256, 0, st>>>(j);
      k_cc_union<<<bs, 256, 0, st>>>(j);
    }
  }
  k_hou_select<<<dim3((j.V + 255) / 256, nlat), 256, 0, st>>>(j);
  k_hou_apply<<<dim3((2 * j.half + 3) / 4, nlat), 256, 0, st>>>(j, g);
  return cudaGetLastError();
}

}  // namespace eagb
