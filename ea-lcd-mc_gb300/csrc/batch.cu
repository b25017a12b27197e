// batch.cu -- persistent batched kernels over a packed (job, block) work list.
#include "batch.cuh"
#include "kernels_dev.cuh"

namespace eagb {

void batch_blocks(const JobDev &j, uint32_t out[KB_COUNT]) {
  const uint32_t nsrb = (uint32_t)(j.ns * j.NR * j.NB);
  const uint32_t nlat = (uint32_t)(j.ns * j.nclust);
  out[KB_SWEEP] = (uint32_t)j.ntiles;
  out[KB_REDUCE] = (nsrb + 255) / 256;
  out[KB_PT] = (uint32_t)(j.ns * ((j.NR + 7) / 8));
  out[KB_MEASURE] = (nsrb + 255) / 256;
  int D, P, nslab;
  if (j.nclust > 0 && slab_shape(j, &D, &P, &nslab) && flip_smem_bytes(j) <= kFlipMaxSmem) {
    out[KB_OVERLAP] = (uint32_t)((2 * j.half + 255) / 256) * nlat;
    out[KB_SLAB] = (uint32_t)nslab * nlat;
    out[KB_MERGE] = (uint32_t)((nslab * j.L * j.L + 255) / 256) * nlat;
    out[KB_COMPRESS] = out[KB_MERGE];
    out[KB_FLIP] = nlat;
  } else {
    out[KB_OVERLAP] = out[KB_SLAB] = out[KB_MERGE] = out[KB_COMPRESS] = out[KB_FLIP] = 0;
  }
}

// Job of work item v: the largest i with pre[i] <= v (pre is non-decreasing).
__device__ __forceinline__ int item_job(const uint32_t *pre, int n, uint32_t v) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pre + mid) <= v) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void dev_slab_shape(const JobDev &j, int &D, int &P, int &nslab) {
  const int S = j.L * j.L;
  D = min(j.Lz, kSlabSites / S);
  P = max(1, min(D, 512 / S));
  nslab = (j.Lz + D - 1) / D;
}

// Next chunk of work for this block.  Every block fetches until it draws a
// chunk index >= the number of chunks, so one launch makes exactly
// nchunks + gridDim.x fetches and atomicInc (which wraps to 0 past its limit)
// leaves the counter at 0 for the next launch.
__device__ __forceinline__ uint32_t fetch_chunk(uint32_t *ctr, uint32_t nchunks, uint32_t *s_v) {
  __syncthreads();
  if (threadIdx.x == 0) *s_v = atomicInc(ctr, nchunks + gridDim.x - 1);
  __syncthreads();
  return *s_v;
}

#define BATCH_LOOP(KIND)                                                                   \
  __shared__ uint32_t s_fetch;                                                             \
  const uint32_t *pre = b.pre[KIND];                                                       \
  const uint32_t total = b.total[KIND], chunk = b.chunk[KIND];                              \
  const uint32_t nchunks = (total + chunk - 1) / chunk;                                     \
  for (;;) {                                                                               \
    const uint32_t c = fetch_chunk(b.ctr + KIND, nchunks, &s_fetch);                       \
    if (c >= nchunks) break;                                                               \
    const uint32_t vend = min(total, (c + 1) * chunk);                                     \
    for (uint32_t v = c * chunk; v < vend; ++v)

__global__ void kb_fill_bits(const __grid_constant__ BatchDev b, int parity) {
  fill_bits_body(b.jobs[blockIdx.x], parity);
}

template <int NR, int KT, bool UPDATE>
__global__ void __launch_bounds__(512, 2) kb_sweep(const __grid_constant__ BatchDev b, int parity, int energy) {
  extern __shared__ __align__(16) unsigned char smem[];
  int staged = -1;  // job whose thresholds are in SMEM
  BATCH_LOOP(KB_SWEEP) {
    const int jb = item_job(pre, b.njobs, v);
    const JobDev jd = b.jobs[jb];  // a copy: no aliasing with the job's arrays
    sweep_body<NR, KT, UPDATE>(jd, (int)(v - __ldg(pre + jb)), parity, energy, smem, jb != staged);
    staged = jb;
    __syncthreads();
  }
  }
}

__global__ void kb_energy_reduce(const __grid_constant__ BatchDev b) {
  BATCH_LOOP(KB_REDUCE) {
    const int jb = item_job(pre, b.njobs, v);
    energy_reduce_body(b.jobs[jb], (int)(v - __ldg(pre + jb)) * blockDim.x + threadIdx.x);
  }
  }
}

__global__ void __launch_bounds__(256) kb_pt(const __grid_constant__ BatchDev b) {
  __shared__ u64 s_ira[8][256];
  __shared__ uint8_t s_wc[8][256];
  BATCH_LOOP(KB_PT) {
    const int jb = item_job(pre, b.njobs, v);
    const JobDev j = b.jobs[jb];
    const int l = (int)(v - __ldg(pre + jb));
    pt_body(j, l % j.ns, l / j.ns, s_ira, s_wc);
    __syncthreads();
  }
  }
}

__global__ void kb_measure(const __grid_constant__ BatchDev b, int itm) {
  BATCH_LOOP(KB_MEASURE) {
    const int jb = item_job(pre, b.njobs, v);
    measure_body(b.jobs[jb], (int)(v - __ldg(pre + jb)) * blockDim.x + threadIdx.x, itm);
  }
  }
}

__global__ void kb_pairs(const __grid_constant__ BatchDev b) {
  const int jb = blockIdx.x * blockDim.x + threadIdx.x;
  if (jb < b.njobs && b.jobs[jb].nclust > 0) pairs_body(b.jobs[jb]);
}

__global__ void kb_overlap(const __grid_constant__ BatchDev b, int g) {
  BATCH_LOOP(KB_OVERLAP) {
    const int jb = item_job(pre, b.njobs, v);
    const JobDev j = b.jobs[jb];
    const int gx = (2 * j.half + 255) / 256, l = (int)(v - __ldg(pre + jb));
    overlap_body(j, g, (l % gx) * 256 + threadIdx.x, (size_t)(l / gx));
  }
  }
}

__global__ void __launch_bounds__(1024, 2) kb_cc_slab(const __grid_constant__ BatchDev b) {
  __shared__ uint32_t lab[kSlabSites];
  __shared__ uint8_t qs[kSlabSites];
  BATCH_LOOP(KB_SLAB) {
    const int jb = item_job(pre, b.njobs, v);
    const JobDev j = b.jobs[jb];
    int D, P, nslab;
    dev_slab_shape(j, D, P, nslab);
    const int l = (int)(v - __ldg(pre + jb));
    cc_slab_body(j, D, P, l % nslab, (size_t)(l / nslab), lab, qs);
    __syncthreads();
  }
  }
}

__global__ void kb_cc_merge(const __grid_constant__ BatchDev b) {
  BATCH_LOOP(KB_MERGE) {
    const int jb = item_job(pre, b.njobs, v);
    const JobDev j = b.jobs[jb];
    int D, P, nslab;
    dev_slab_shape(j, D, P, nslab);
    const int gx = (nslab * j.L * j.L + 255) / 256, l = (int)(v - __ldg(pre + jb));
    cc_merge_body(j, D, nslab, (l % gx) * 256 + threadIdx.x, (size_t)(l / gx));
  }
  }
}

__global__ void kb_cc_compress(const __grid_constant__ BatchDev b) {
  BATCH_LOOP(KB_COMPRESS) {
    const int jb = item_job(pre, b.njobs, v);
    const JobDev j = b.jobs[jb];
    int D, P, nslab;
    dev_slab_shape(j, D, P, nslab);
    const int gx = (nslab * j.L * j.L + 255) / 256, l = (int)(v - __ldg(pre + jb));
    cc_compress_body(j, D, nslab, (l % gx) * 256 + threadIdx.x, (size_t)(l / gx));
  }
  }
}

__global__ void __launch_bounds__(512) kb_flip(const __grid_constant__ BatchDev b, const __grid_constant__ UTable u,
                                               int g) {
  extern __shared__ uint32_t s_flip[];
  BATCH_LOOP(KB_FLIP) {
    const int jb = item_job(pre, b.njobs, v);
    const JobDev jd = b.jobs[jb];
    flip_body(jd, u.u[jb], g, (size_t)(v - __ldg(pre + jb)), s_flip + 64, reinterpret_cast<int *>(s_flip));
    __syncthreads();
  }
  }
}

// ---------------------------------------------------------------------------
// Launchers: persistent grids of (SMs x resident blocks), never more blocks
// than items.
// ---------------------------------------------------------------------------
static int g_sms = 0;

static unsigned grid_for(uint32_t items, int per_sm) {
  const uint32_t cap = (uint32_t)(g_sms > 0 ? g_sms : 1) * (uint32_t)per_sm;
  return items < cap ? (items ? items : 1) : cap;
}

static uint32_t chunks(const BatchDev &b, int k) { return (b.total[k] + b.chunk[k] - 1) / b.chunk[k]; }

template <int NR, int KT>
static cudaError_t sweep_setup() {
  // 227 KB per block, less the kernel's static SMEM (the fetch slot)
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kb_sweep<NR, KT, true>);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kb_sweep<NR, KT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              227 * 1024 - (int)fa.sharedSizeBytes);
}

cudaError_t batch_setup(int NR, int KT) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kb_flip, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFlipMaxSmem);
  if (e != cudaSuccess) return e;
  switch (NR * 100 + KT) {
    case 801: return sweep_setup<8, 1>();
    case 802: return sweep_setup<8, 2>();
    case 804: return sweep_setup<8, 4>();
    case 402: return sweep_setup<4, 2>();
    case 404: return sweep_setup<4, 4>();
    case 408: return sweep_setup<4, 8>();
    case 204: return sweep_setup<2, 4>();
    case 208: return sweep_setup<2, 8>();
    case 216: return sweep_setup<2, 16>();
    default: return cudaErrorInvalidValue;
  }
}

int batch_sweep_smem(int NR, int KT, int NBmax) { return (int)sweep_smem_for(NBmax, NR, KT); }

cudaError_t batch_fill_bits(const BatchDev &b, int parity, cudaStream_t st) {
  kb_fill_bits<<<b.njobs, 64, 0, st>>>(b, parity);
  return cudaGetLastError();
}

template <int NR, int KT>
static cudaError_t batch_sweep_t(const BatchDev &b, int NBmax, int parity, bool energy, bool update, cudaStream_t st) {
  if (!b.total[KB_SWEEP]) return cudaSuccess;
  if (update) {
    const int sm = batch_sweep_smem(NR, KT, NBmax);
    const int per_sm = sm > 0 ? (int)((228 * 1024) / (sm + 1024)) : 4;
    kb_sweep<NR, KT, true><<<grid_for(chunks(b, KB_SWEEP), per_sm < 1 ? 1 : (per_sm > 4 ? 4 : per_sm)), 512, sm, st>>>(
        b, parity, energy ? 1 : 0);
  } else {
    kb_sweep<NR, KT, false><<<grid_for(chunks(b, KB_SWEEP), 4), 512, KT * 8 * 4, st>>>(b, parity, 1);
  }
  return cudaGetLastError();
}

cudaError_t batch_sweep(const BatchDev &b, int NR, int KT, int NBmax, int parity, bool energy, bool update,
                        cudaStream_t st) {
  switch (NR * 100 + KT) {
    case 801: return batch_sweep_t<8, 1>(b, NBmax, parity, energy, update, st);
    case 802: return batch_sweep_t<8, 2>(b, NBmax, parity, energy, update, st);
    case 804: return batch_sweep_t<8, 4>(b, NBmax, parity, energy, update, st);
    case 402: return batch_sweep_t<4, 2>(b, NBmax, parity, energy, update, st);
    case 404: return batch_sweep_t<4, 4>(b, NBmax, parity, energy, update, st);
    case 408: return batch_sweep_t<4, 8>(b, NBmax, parity, energy, update, st);
    case 204: return batch_sweep_t<2, 4>(b, NBmax, parity, energy, update, st);
    case 208: return batch_sweep_t<2, 8>(b, NBmax, parity, energy, update, st);
    case 216: return batch_sweep_t<2, 16>(b, NBmax, parity, energy, update, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t batch_energy_reduce(const BatchDev &b, cudaStream_t st) {
  if (b.total[KB_REDUCE]) kb_energy_reduce<<<grid_for(chunks(b, KB_REDUCE), 8), 256, 0, st>>>(b);
  return cudaGetLastError();
}

cudaError_t batch_pt(const BatchDev &b, cudaStream_t st) {
  if (b.total[KB_PT]) kb_pt<<<grid_for(chunks(b, KB_PT), 8), 256, 0, st>>>(b);
  return cudaGetLastError();
}

cudaError_t batch_measure(const BatchDev &b, int itm, cudaStream_t st) {
  if (b.total[KB_MEASURE]) kb_measure<<<grid_for(chunks(b, KB_MEASURE), 8), 256, 0, st>>>(b, itm);
  return cudaGetLastError();
}

cudaError_t batch_pairs(const BatchDev &b, cudaStream_t st) {
  kb_pairs<<<(b.njobs + 127) / 128, 128, 0, st>>>(b);
  return cudaGetLastError();
}

cudaError_t batch_houdayer_group(const BatchDev &b, const UTable &u, int g, cudaStream_t st) {
  if (!b.total[KB_SLAB]) return cudaSuccess;
  kb_overlap<<<grid_for(chunks(b, KB_OVERLAP), 8), 256, 0, st>>>(b, g);
  const int per_sm = b.slab_threads > 0 ? 2048 / b.slab_threads : 1;
  kb_cc_slab<<<grid_for(chunks(b, KB_SLAB), per_sm < 1 ? 1 : per_sm), b.slab_threads, 0, st>>>(b);
  kb_cc_merge<<<grid_for(chunks(b, KB_MERGE), 8), 256, 0, st>>>(b);
  kb_cc_compress<<<grid_for(chunks(b, KB_COMPRESS), 8), 256, 0, st>>>(b);
  kb_flip<<<grid_for(chunks(b, KB_FLIP), 4), 512, b.flip_smem, st>>>(b, u, g);
  return cudaGetLastError();
}

}  // namespace eagb
