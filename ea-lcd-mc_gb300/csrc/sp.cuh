// sp.cuh -- sample-packed layout: 64 disorder samples per 64-bit word (bit b =
// sample b of the word), for tubes of any L >= 2 and Lz >= 2 and any number of
// replicas.  The reference's multispin layout packs 64 sub-blocks of ONE
// sample per word and so needs L and Lz multiples of 8 (PROGRAM/include/
// header.h:41-47); here every word of a site holds the same site of 64
// samples, so the lattice is a plain site list with a neighbour table and a
// proper colouring (2 colours for bipartite tubes, more otherwise).
//
// The update arithmetic is the reference's: Philox4x32-10 random words turned
// into heat-bath bits through the temperature's 64-bit thresholds
// (main.cu:994-1150), the bit-sliced local field and flip mask
// (main.cu:1474-1506), 6 bond slots per site with the reference's fake bond
// on the open z planes (ini.c:551-641, main.cu:1460-1472), E = 3V - 2 x
// unsatisfied bonds (main.cu:1379) and the tempering rule of upd.c:3-48.
// Each temperature slot has a fixed beta; tempering swaps move the
// configurations of the accepted samples between slots (lane masks).
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include "eagb.h"

namespace eagb {

// Lattice graph of the sample-packed layout (host).
struct SpGraph {
  int L = 0, Lz = 0, bc = 0, V = 0, ncol = 0;
  std::vector<int32_t> nb;         // [V][6] neighbour site of each bond slot (+x,+y,+z,-x,-y,-z)
  std::vector<int32_t> mate;       // [V][6] half-edge index p*6+slot' of the other end
  std::vector<uint8_t> colour;     // [V]
  std::vector<int32_t> col_off;    // [ncol+1]
  std::vector<int32_t> col_sites;  // [V] sites grouped by colour, ascending
};
bool sp_graph(int L, int Lz, int bc, SpGraph &g);
void sp_couplings(const SpGraph &g, int nwords, uint64_t seed_J, uint64_t *J);
void sp_spins(const SpGraph &g, int nwords, int NR, int NB, uint64_t seed_u, uint64_t *S);

// Device view of a sample-packed job (kernel parameter).
struct SpDev {
  int L, Lz, V, bc, NB, NR, nw, ncol, kt;
  int echunk;                        // sites per thread of the energy count
  int esites, epair;                 // sites the count walks: all V, or (epair = 1) the colour-1 sites, counted twice
  int cthreads;                      // block size of the one-job cluster labelling
  int pgrid;                         // > 0: one-job colour passes as the per-item pass on this many CTAs
  int col_off[9];                    // colour c owns col_sites[col_off[c] .. col_off[c+1])
  const int32_t *nb;                 // [V][6]
  const int32_t *col_sites;          // [V]
  unsigned long long *S;             // [nw][V][NR][NB] spin words
  const unsigned long long *J;       // [nw][V][6] coupling words
  const unsigned long long *cum;     // [NB][256] thresholds
  const uint16_t *pre;               // [NB][256] 8-bit pre-search
  const uint8_t *pre11;              // [NB][2064] 11-bit pre-search (the per-item pass)
  uint4 *ctr;                        // [NR] Philox counters of the current pass
  const uint32_t *keys;              // [NR]
  ea_hq *prc;                        // [NR]
  ea_xoshiro *xo;                    // [NR]
  long long *iter;                   // colour-pass counter
  uint32_t jobid;
  int32_t *U2;                       // [nw][64][NR][NB] unsatisfied half-edges (twice the bonds)
  int32_t *E;                        // [nw][64][NR][NB] energy of the configuration at each slot
  uint8_t *perm;                     // [nw][64][NR][NB] replica-local id of the configuration at each slot
  uint32_t *acc;                     // [nw][64][NR][NB-1] accepted swaps
  unsigned long long *M;             // [nw][NR][NB-1] lanes that swapped in the last tempering step
  const double *betas;               // [NB] descending
  const double *exptab;              // host-libm exp of the tempering exponents
  const int32_t *expoff;             // [NB]
  unsigned long long *ptstep;        // tempering steps so far
  unsigned long long pt_seed;
  double *avgE;                      // [nw][64][NR][NB]
  // Houdayer move
  ea_hq *rc;                         // replica-pair generator (random_c)
  int32_t *pairs;                    // [2 groups][2]
  unsigned long long *Q;             // [nw][nclust][V] overlap words s_r1 ^ s_r2
  unsigned long long *move;          // cluster moves so far
  int nclust;
  uint32_t *cscratch;                // labelling arrays of lattices above kSpClusterMaxV, per CTA
  int slabD;                         // > 0: such lattices labelled in slabs of slabD z planes (one-job path)
  uint32_t *slab_lab;                // [nw*nclust*8 units][8][V] labels of the slab path
  uint8_t *slab_coin;                // [units][V] roots' coins (one bit a sample)
  // exact enumeration
  unsigned long long *dos;           // [nw][64][6V+1] states per energy (E = -3V..3V)
};

// Largest lattice of the one-CTA cluster labelling in SMEM (7 bytes per
// site: label, 8 samples' overlap and flip bits, bond mask); larger ones use
// a global scratch region of sp_cluster_words(V) words per CTA.
constexpr int kSpClusterMaxV = 32768;
// Lattices up to this size are labelled 4 samples at a time (22 bytes of
// SMEM per site; 512 bytes left for static SMEM).
constexpr int kSpCluster4MaxV = 10500;
__host__ __device__ inline size_t sp_cluster_words(int V) { return ((size_t)V * 7 + 15) / 16 * 4; }

int sp_kt(int NB, int NR, int nsites_colour);
int sp_slab_planes(int L, int Lz, int nw, int nclust);
int sp_energy_chunk(const SpDev &d);
size_t sp_sweep_smem(int NB, int NR, int kt);
size_t sp_items_smem(int NB);
int sp_items_grid(int NB);
cudaError_t sp_setup();
cudaError_t sp_launch_pass(const SpDev &d, int colour, int off, int n, cudaStream_t st);
cudaError_t sp_launch_energy(const SpDev &d, cudaStream_t st);
cudaError_t sp_launch_pt(const SpDev &d, cudaStream_t st);
cudaError_t sp_launch_permute(const SpDev &d, cudaStream_t st);
cudaError_t sp_launch_houdayer(const SpDev &d, cudaStream_t st);
cudaError_t sp_launch_measure_u2(const SpDev &d, bool from_e, cudaStream_t st);
cudaError_t sp_launch_dos(const SpDev &d, cudaStream_t st);
cudaError_t sp_launch_exact(const SpDev &d, const double *betas, int nbeta, double *meanE, cudaStream_t st);

// Batched sample-packed kernels: one launch per kernel kind for every job of
// a batch, block b of a launch working for the job j with pre[j] <= b < pre[j+1].
enum {
  SPB_PASS0 = 0, SPB_PASS1, SPB_PASS2, SPB_PASS3,  // colour passes (jobs with that colour)
  SPB_ZERO, SPB_ENERGY, SPB_PT, SPB_PERMUTE, SPB_MEASURE,
  SPB_OVL0, SPB_OVL1, SPB_CL0, SPB_CL1, SPB_FL0, SPB_FL1,  // Houdayer, per replica group
  SPB_COUNT
};
constexpr int kSpBatchMaxColours = 4;
struct SpBatchDev {
  const SpDev *jobs;
  int njobs;
  const uint32_t *pre[SPB_COUNT];
  uint32_t total[SPB_COUNT];
  int pass_smem, perm_smem, cluster_smem;  // dynamic SMEM of the largest job
  int cluster_threads;                      // block size of the labelling
};
void sp_batch_blocks(const SpDev &d, bool cluster, uint32_t out[SPB_COUNT]);

// Persistent bin kernel (k_sp_persist): whole bins of the jobs of a work
// list in one cooperative launch.
struct SpPersistDev {
  SpBatchDev b;
  int itmax, houfr, mesfr, ptfr, cluster, ncol_max;
  unsigned long long *bar;  // arrivals at the grid barrier (zeroed by sp_launch_persist)
  int *err;                 // barrier waits that gave up (zero at set-up; read by the host)
};
int sp_persist_grid(const SpBatchDev &b, size_t smem);
cudaError_t sp_launch_persist(const SpPersistDev &p, int grid, size_t smem, cudaStream_t st);

// Resident bin kernel (sp_resident.cu): bins without cluster moves of a job
// whose words fit in the shared memory of one thread-block cluster.  CTA c
// of the cluster owns the sites [c*nslm, (c+1)*nslm); the random words of
// the launch's sweeps are drawn beforehand by k_sp_draw.
constexpr int kResMaxCta = 16;
constexpr int kResMinBlock = 4;  // fewest sweeps between cluster moves for a resident launch to pay
constexpr int kResMaxColours = 8;
struct SpResDev {
  SpDev d;
  const unsigned long long *R;  // [sweep][colour blocks: 3 planes x NR x NB x sites of the colour]
  const unsigned long long *X;  // [tempering step][word x replica][pair][sample] FNORM * u as bits
  int nit, nsweep, houfr, mesfr, ptfr;  // iterations and sweeps of this launch, the cadence
  int pair_energy;               // count the energy in the last colour pass (see ea_sp::pair_energy)
  int measure;                   // add the energies to the bin's sums after each iteration (no cluster moves)
  int ncta, nslm, upc;           // CTAs, sites per CTA, tempering chains (word, replica) per CTA
  int ntab;                      // exp table entries staged in SMEM (0: read from global memory)
  int lpc_count, lpc_energy;     // lanes per column of the counts in the last pass / the energy phase (8, 16, 32)
  int kr[kResMaxCta + 1][kResMaxColours];  // first index into colour k's site list of CTA c's sites
};
struct SpResPlan {
  int ncta = 0, nslm = 0, upc = 0, ntab = 0, npl = 0, lpc_count = 32, lpc_energy = 32;
  size_t smem = 0;
  int kr[kResMaxCta + 1][kResMaxColours] = {};
};
// Fills `pl` and returns true when the job can run resident (colours, SMEM,
// a co-resident cluster); col_sites: the host's colour-ordered site list,
// ntab: entries of the job's exp table.
bool sp_res_plan(const SpDev &d, const int32_t *col_sites, int ntab, SpResPlan &pl);
bool sp_res_fits(int L, int Lz, int nw, int NR, int NB);  // the size test of sp_res_plan alone
// Sweeps of random words one resident launch holds: whole iterations of the
// cadence, up to 16 MB, at least one iteration; with cluster moves one block
// of houfr x ptfr sweeps (at least kResMinBlock) between two moves; 0 when
// that exceeds 256 MB or the block is shorter (the resident kernel does not
// take such bins).
size_t sp_res_launch_sweeps(size_t V, size_t G, const ea_cadence *cad);
cudaError_t sp_res_setup();
// One launch's worth: the counters of npass colour passes, their random
// words, then the resident kernel over p.nit iterations.
cudaError_t sp_res_chunk(const SpResDev &p, const SpResPlan &pl, int npass, uint4 *ctrs, cudaStream_t st);
cudaError_t sp_batch_setup();
cudaError_t sp_batch_sweep(const SpBatchDev &b, int ncol_max, cudaStream_t st);
cudaError_t sp_batch_tempering(const SpBatchDev &b, cudaStream_t st);
cudaError_t sp_batch_houdayer(const SpBatchDev &b, cudaStream_t st);
cudaError_t sp_batch_measure(const SpBatchDev &b, bool from_e, cudaStream_t st);

}  // namespace eagb
