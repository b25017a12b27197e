// kernels.cuh -- device-side job descriptor and kernel launchers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "eagb.h"

namespace eagb {

// Division by a value fixed at set-up, exact for every 32-bit numerator: one
// multiply-high, an add and two shifts (the round-up method for unsigned
// division by invariant integers, Granlund & Montgomery, PLDI 1994).
struct FastDiv {
  uint32_t d = 1, m = 1, s1 = 0, s2 = 0;
  void set(uint32_t dd) {
    d = dd ? dd : 1;
    int l = 0;
    while ((1ull << l) < d) ++l;
    m = (uint32_t)((((1ull << 32) * ((1ull << l) - d)) / d) + 1);
    s1 = l < 1 ? l : 1;
    s2 = l > 1 ? l - 1 : 0;
  }
#ifdef __CUDACC__
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    const uint32_t t = __umulhi(m, n);
    return (t + ((n - t) >> s1)) >> s2;
  }
  __device__ __forceinline__ uint32_t mod(uint32_t n) const { return n - div(n) * d; }
#endif
};

// Everything a kernel needs about one job, by value (kernel parameter).
// All arrays live in device memory, in the reference's layouts.
struct JobDev {
  int NB, NR, ns, half, msc_l, msc_s, msc_lz, L, Lz, V, bc;
  unsigned long long *spins;        // [s][parity][clone][half][rep]
  const unsigned long long *J;      // [s][parity][dir][half]
  const int32_t *nbidx;             // [parity][dir][half]
  const uint8_t *nbflag;            // [parity][half]
  const unsigned long long *cum;    // [NB][256] thresholds
  const uint16_t *pre;              // [NB][256] 8-bit pre-search
  uint8_t *wctb, *wbtc;             // [s][rep][NB]
  uint4 *ctr;                       // [NR] Philox counters of the current half-sweep
  const uint32_t *keys;             // [NR]
  ea_hq *prc;                       // [NR]
  ea_xoshiro *xo;                   // [NR]
  long long *iter;                  // half-sweep counter (device scalar)
  uint32_t jobid;
  int32_t *epart;                   // [ntiles][s][clone][rep] energy partial sums
  int ntiles, kt;
  int32_t *E;                       // [s][rep][clone]
  // parallel tempering
  ea_hq *pt;                        // [s][rep]
  const double *betas;              // [NB]
  const double *exptab;             // glibc exp table
  const int32_t *expoff;            // [NB]
  double *acc, *att, *accraw;       // [s][rep][NB-1]
  unsigned long long *inexact;      // decisions decided outside the table (u == 0)
  // measurements
  double *avgE;                     // [s][rep][NB]
  uint8_t *hist;                    // [s][rep][maxit][NB]
  int maxit_trw;
  // Houdayer
  ea_hq *rc;
  int32_t *pairs;                   // [2 groups][2]
  unsigned long long *Q;            // [s][nclust][2][half] overlap words
  uint32_t *label;                  // [s][nclust][V] natural order
  uint32_t *sel;                    // [s][nclust][V / 32] cluster selection bits, natural order
  const double *U;                  // [s][NB][V] uniforms of the current group
  int nclust;
  // x coordinate against which site 0 tests its periodic -x bond.  The
  // reference computes (ltid-1+nx)%nx with a 32-bit ltid (HoudayerXEA.cu:96),
  // i.e. (2^32-1+L) mod L, which differs from L-1 unless L is a power of two;
  // the union itself still joins sites 0 and L-1 (HoudayerXEA.cu:288).
  int cc_xq;
  // dividers of the site <-> multispin-word maps
  FastDiv fd_L, fd_S, fd_ml, fd_mlz, fd_hl, fd_nclust;
};

constexpr int kSlabSites = 8192;        // sites of a slab held in SMEM
constexpr int kSlabMaxPerThread = 16;   // sites a thread of the slab labelling owns

// Shared memory of the one-CTA-per-lattice selection and flip (V/8 bytes of
// selection bits + the 64 bit offsets); larger lattices take the two-kernel
// path (global selection bits).
constexpr size_t kFlipMaxSmem = 200 * 1024;
size_t flip_smem_bytes(const JobDev &j);

// Slab labelling shape of a job: planes per slab D, planes per pass P and the
// number of slabs; false when its planes need the generic labelling.
bool slab_shape(const JobDev &j, int *D, int *P, int *nslab);

// Fills the dividers of j from its sizes (nclust included).
void set_dividers(JobDev &j);

// Tile width (half-sites per CTA) of the fused sweep kernel.
int sweep_kt(const JobDev &j);
size_t sweep_smem_bytes(const JobDev &j);
// Dynamic SMEM of a fused half-sweep CTA: the random triples of the tile
// (3 x NB x KT x NR words), the pre-search tables (NB x 256 x 2 B) and the
// tile's neighbour records (KT x 8 ints).
inline size_t sweep_smem_for(int NB, int NR, int KT) {
  return (size_t)3 * NB * KT * NR * 8 + (size_t)NB * 256 * 2 + (size_t)KT * 8 * 4;
}

cudaError_t launch_fill_bits(const JobDev &j, int parity, cudaStream_t st);
cudaError_t launch_sweep(const JobDev &j, int parity, bool energy, cudaStream_t st);
cudaError_t launch_energy(const JobDev &j, cudaStream_t st);
cudaError_t launch_energy_reduce(const JobDev &j, cudaStream_t st);
cudaError_t launch_pt(const JobDev &j, cudaStream_t st);
cudaError_t launch_measure(const JobDev &j, int itm, cudaStream_t st);
cudaError_t launch_houdayer_pairs(const JobDev &j, cudaStream_t st);
cudaError_t launch_houdayer_group(const JobDev &j, int group, cudaStream_t st);

}  // namespace eagb
