/*
 * ea_oracle.h -- CPU restatement of the EA-LCD-MC simulation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * in ea-lcd-mc_gb300/ is compared against.  Only tests/, __graft_entry__.smoke()
 * and the cpu_baseline / reference legs of bench.py may load it.  The product
 * never links, loads or calls anything under oracle/.
 *
 * Every function restates one piece of the reference (paths relative to the
 * reference project root, PROGRAM/...).  Parity is pinned by
 * tests/golden/ (fixtures produced by the reference's own host code compiled
 * from its sources, and by the reference CUDA binary run on a GB300).
 *
 * All geometry is runtime (the reference fixes it at compile time through
 * L, Lz, NBETAS, NR macros, PROGRAM/include/header.h:14-66).
 */
#ifndef EA_ORACLE_H
#define EA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parisi-Rapuano + congruential 64-bit generator, PROGRAM/include/random_generator.h:31-38 */
typedef struct {
  uint64_t ira[256];
  uint64_t PR;
  uint64_t zseed;
  uint64_t final;
  uint8_t ip, ip1, ip2, ip3;
  uint8_t padding[4];
} or_hq;

/* xoshiro256++, PROGRAM/include/random_generator.h:41-46 */
typedef struct {
  uint64_t s[4];
  uint64_t t;
  uint64_t final;
} or_xo;

enum { OR_PBC = 0, OR_OBC = 1, OR_OBC_WEAK = 2, OR_OBC_STRONG = 3 };

/* Geometry of one tube L x L x Lz in the reference multispin layout. */
typedef struct {
  int L, Lz, NB, NR, nbits, bc;
  int msc_l, msc_lz, msc_s, msc_v, half, V;
} or_geom;

int or_geom_init(or_geom *g, int L, int Lz, int NB, int NR, int nbits, int bc);

/* ---- host generators ---------------------------------------------------- */
uint64_t or_hq_next(or_hq *u);
void or_hq_init(or_hq *u, uint64_t seed);
uint64_t or_xo_next(or_xo *u);
void or_inicia_generadores(or_hq *prc, or_xo *xo, uint32_t *key, uint64_t seed);
void or_seeds_from_one(uint64_t seed, uint64_t *list, int nseeds);

/* All seeds and generator states of one run (reference Init_Random + seeds). */
typedef struct {
  uint64_t seeds_J[32], seeds_u[32], seeds_MC[64];
  uint64_t seed_cluster;
} or_seeds;

void or_generate_seed_vectors(uint64_t master_J, uint64_t master_u, uint64_t master_MC,
                              const int *list_samples, int nbits, int NR, or_seeds *out);
void or_init_random(const or_seeds *sd, const int *list_samples, int nbits, int NR,
                    or_hq *prc /*[NR]*/, or_xo *xo /*[NR]*/, uint32_t *keys /*[NR]*/,
                    or_hq *pt /*[nbits*NR]*/, or_hq *rc);

/* ---- geometry, spins, couplings ------------------------------------------ */
void or_tables(const or_geom *g, int32_t *neig /*[2][6][half]*/, uint8_t *rot /*[2][half]*/,
               uint32_t *bianchi /*[half]*/, uint32_t *neri /*[half]*/);
void or_init_spins(const or_geom *g, uint64_t seed_u, uint8_t *uu /*[NR][NB][V]*/);
void or_pack_spins(const or_geom *g, const uint8_t *uu, uint64_t *even, uint64_t *odd);
void or_unpack_spins(const or_geom *g, const uint64_t *even, const uint64_t *odd, uint8_t *uu);
int or_init_couplings(const or_geom *g, uint64_t seed_J, uint8_t *J6 /*[6][V]: x,y,z,mx,my,mz*/);
void or_pack_couplings(const or_geom *g, const uint8_t *J6, uint64_t *Jw /*[2][6][half]*/);

/* ---- Metropolis random words ---------------------------------------------- */
void or_fill_bits(or_hq *prc, or_xo *xo, int NR, uint64_t iter, uint32_t jobid,
                  uint32_t *ctr /*[NR][4]*/);
void or_rnd_triple(const uint32_t ctr[4], uint32_t key, uint32_t tid,
                   const uint64_t *cum /*[256]*/, uint64_t out[3]);
int or_lut_search(uint64_t R, const uint64_t *cum);

/* One checkerboard half-sweep of parity p for every sample (d_gen_rndbits_cuda +
 * d_oneMCstepBN_multisample).  spins: [nbits][2][NB][half][NR]; Jw: [nbits][2][6][half];
 * wbtc: [nbits][NR][NB] (beta index of each clone); cum: [NB][256]. */
void or_half_sweep(const or_geom *g, uint64_t *spins, const uint64_t *Jw,
                   const uint8_t *wbtc, const uint32_t *ctr, const uint32_t *keys,
                   const uint64_t *cum, int parity, int nthreads);

/* d_computeEne: energies [nbits][NR][NB] (clone index). */
void or_energy(const or_geom *g, const uint64_t *spins, const uint64_t *Jw, int32_t *E);
/* med.c calculate_scalar_energy on unpacked spins of one (replica, clone). */
int or_scalar_energy(const or_geom *g, const uint8_t *u /*[V]*/, const uint8_t *J6);

/* upd.c Parallel_Tempering for one (sample, replica). */
void or_parallel_tempering(or_hq *p, uint8_t *wctb, uint8_t *wbtc, const int32_t *E,
                           const double *betas, int NB, double *acc, double *att,
                           double *accraw);

/* Houdayer: pair choice (main.cu:409-421). */
void or_houdayer_pair(or_hq *rc, int NR, int g, int *r1, int *r2);
/* Overlap, cluster labelling, flip and apply for one replica pair over every
 * sample.  U: [nbits][NB][V] uniforms of this cluster step.  nclust: number of
 * beta indices (coldest first) that take part (lround(0.5*NB) in the reference). */
void or_houdayer_group(const or_geom *g, uint64_t *spins, const uint8_t *wctb, int r1, int r2,
                       const double *U, int nclust, int ref_quirk);
/* Labels only (for tests): root[V] = minimum site index of the equal-q cluster.
 * ref_quirk != 0 reproduces the reference's test of site 0's x-wrap bond. */
void or_cluster_roots(const or_geom *g, const uint8_t *q /*[V]*/, uint32_t *root, int ref_quirk);

/* ---- LUT (create_LUT.c) ----------------------------------------------------- */
/* Cumulative thresholds and the reference file layout of one beta.  Returns 0 on
 * success, -1 when the oracle was compiled without quad precision. */
int or_lut_beta(double beta, int nbits_pre, uint64_t *cum /*[256]*/, uint32_t *umbrales /*[512]*/,
                uint32_t *prebusqueda /*[(1<<nbits_pre)/2]*/);

/* ---- Whole run ---------------------------------------------------------------- */
typedef struct {
  int nbin, itcut, itmax, houfr, mesfr, ptfr;
  uint32_t jobid;
  int cluster;     /* 0: NO_CLUSTER */
  int nclust;      /* beta indices in the Houdayer move */
  int nthreads;
  int cluster_exact; /* 1: test site 0's x-wrap bond correctly (not the reference's behaviour) */
} or_run_cfg;

/* Complete mutable state of a run (host view). */
typedef struct {
  or_geom g;
  uint64_t *spins;          /* [nbits][2][NB][half][NR] */
  uint64_t *Jw;             /* [nbits][2][6][half] */
  uint8_t *wctb, *wbtc;     /* [nbits][NR][NB] */
  int32_t *E;               /* [nbits][NR][NB] last measured, clone index */
  double *acc, *att, *accraw; /* [nbits][NR][NB-1] */
  double *avgE;             /* [nbits][NR][NB] beta order, summed over it */
  uint8_t *hist;            /* [nbits][NR][maxit_trw][NB] */
  or_hq *prc; or_xo *xo; uint32_t *keys; or_hq *pt; or_hq rc;
  uint64_t cuda_rng_offset;
  uint64_t seed_cluster;
  double *betas;            /* [NB] */
  uint64_t *cum;            /* [NB][256] */
  int frec_trw, maxit_trw;
  /* cuRAND host generator, created at the first cluster move with
   * (seed_cluster, cuda_rng_offset) and then kept, as the reference keeps its
   * device generator for the life of the process (HoudayerXEA.cu:174-178).
   * A fresh generator at offset n does not continue one that produced n numbers. */
  void *curand_gen;
} or_state;

void or_state_release(or_state *st);

/* Advance one bin (the body of the ibin loop, main.cu:142-230): Monte Carlo,
 * energy, PT, Houdayer, averages and history.  *iter is the half-sweep counter.
 * Uniforms are drawn with the cuRAND host XORWOW generator (seed, offset). */
int or_run_bin(or_state *st, const or_run_cfg *cfg, uint64_t *iter);
int or_curand_host(uint64_t seed, uint64_t offset, uint64_t n, double *out);

/* Sample-packed layout (sp_oracle.c): 64 samples per word, any L, Lz. */
void or_sp_pass(int V, int NR, int NB, int nw, const int32_t *nb, const int32_t *sites, int nsites,
                const uint32_t *ctr, const uint32_t *keys, const uint64_t *cum, const uint64_t *J, uint64_t *S);
void or_sp_energy(int V, int NR, int NB, int nw, const int32_t *nb, const uint64_t *J, const uint64_t *S,
                  int32_t *U2);
void or_sp_pt(int V, int NR, int NB, int nw, const double *betas, const double *exptab, const int32_t *expoff,
              uint64_t step, uint64_t seed, const int32_t *U2, int32_t *E, uint8_t *perm, uint32_t *acc,
              uint64_t *masks, uint64_t *S);
void or_sp_dos(int V, const int32_t *nb, const uint64_t *J, int w, int lane, uint64_t *hist);
void or_sp_cluster(int V, int NR, int NB, int nw, const int32_t *nb, int nclust, int g, int r1, int r2,
                   uint64_t move, uint64_t key, uint64_t *S);

#ifdef __cplusplus
}
#endif
#endif
