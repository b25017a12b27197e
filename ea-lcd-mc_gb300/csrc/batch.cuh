// batch.cuh -- persistent batched kernels: one launch serves every job of a
// batch (different L, Lz, boundary condition, NB and sample count) by walking
// a packed work list of (job, block) items.  Each item runs the same device
// body as the one-job kernel, so a job's words are the same alone and in a
// batch.
#pragma once
#include "kernels.cuh"

namespace eagb {

// Work-list kinds: the blocks of one job for each one-job kernel.
enum { KB_SWEEP = 0, KB_REDUCE, KB_PT, KB_MEASURE, KB_OVERLAP, KB_SLAB, KB_MERGE, KB_COMPRESS, KB_FLIP, KB_COUNT };

constexpr int kBatchMaxJobs = 1024;

// Device view of a batch (kernel parameter).  pre[k] is the exclusive prefix
// sum over jobs of their block counts for kind k ([njobs + 1] entries).
// Blocks take work from ctr[k] in chunks of chunk[k] items; the counter
// returns to 0 by itself at the end of every launch (see item fetching in
// batch.cu), so launches replay from a CUDA graph without resets.
struct BatchDev {
  const JobDev *jobs;
  int njobs;
  const uint32_t *pre[KB_COUNT];
  uint32_t total[KB_COUNT];
  uint32_t chunk[KB_COUNT];
  uint32_t *ctr;     // [KB_COUNT] work counters
  int slab_threads;  // block size of the slab labelling (largest L^2 * P)
  int flip_smem;     // dynamic SMEM of the flip (largest lattice)
};

// Uniforms of the current group for every job (kernel parameter).
struct UTable {
  const double *u[kBatchMaxJobs];
};

// Blocks of job j for each kind (the one-job launch geometry, flattened).
void batch_blocks(const JobDev &j, uint32_t out[KB_COUNT]);

int batch_sweep_smem(int NR, int KT, int NBmax);
// Kernel attributes and device figures the launchers use; called before any
// launch (and so before a stream capture).
cudaError_t batch_setup(int NR, int KT);
cudaError_t batch_fill_bits(const BatchDev &b, int parity, cudaStream_t st);
cudaError_t batch_sweep(const BatchDev &b, int NR, int KT, int NBmax, int parity, bool energy, bool update,
                        cudaStream_t st);
cudaError_t batch_energy_reduce(const BatchDev &b, cudaStream_t st);
cudaError_t batch_pt(const BatchDev &b, cudaStream_t st);
cudaError_t batch_measure(const BatchDev &b, int itm, cudaStream_t st);
cudaError_t batch_pairs(const BatchDev &b, cudaStream_t st);
cudaError_t batch_houdayer_group(const BatchDev &b, const UTable &u, int g, cudaStream_t st);

}  // namespace eagb
