/*
 * eagb.h -- C ABI of the GB300-native EA-LCD-MC simulation library (libeagb.so).
 *
 * One context = one simulation job as the reference runs it in one process:
 * `nsamples` disorder samples ("nbits" on the reference command line) of an
 * L x L x Lz tube, NR replicas and NB temperatures, in the reference's
 * multispin layout (64 spatial sub-blocks per 64-bit word).  The context owns
 * all device memory and one CUDA stream; host buffers are caller-owned and
 * only copied.  Every function returns EA_OK (0) or a negative EA_ERR_*
 * code and never exits the process; ea_last_error() describes the last
 * failure of the calling thread.  One context must not be used by two host
 * threads at the same time.
 *
 * Layouts (identical to the reference's host arrays):
 *   spins    even/odd arrays [clone][half][replica] uint64 (PROGRAM/src/ini.c:339-383)
 *   couplings Jw[parity][dir][half] uint64, dir = +x,+y,+z,-x,-y,-z (ini.c:672-730)
 *   permutations which_clon_this_beta[sample][replica][beta] (header.h:153-154)
 *   energies [sample][replica][clone] int32, E = 3V - 2 * unsatisfied bonds (main.cu:1379)
 *   thresholds cum[beta][256]: the 64-bit cumulative thresholds of the LUT
 *             file, 'umbrales' (PROGRAM/input/create_LUT.c:301-326)
 */
#ifndef EAGB_H
#define EAGB_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EA_VERSION 100

enum {
  EA_OK = 0,
  EA_ERR_ARG = -1,     /* invalid argument or geometry */
  EA_ERR_CUDA = -2,    /* CUDA runtime error */
  EA_ERR_NOMEM = -3,   /* device or host allocation failed */
  EA_ERR_STATE = -4,   /* call out of order (e.g. run before inputs are set) */
  EA_ERR_CURAND = -5,  /* cuRAND error */
  EA_ERR_IO = -6,      /* file I/O or format error */
  EA_ERR_INEXACT = -7  /* a PT decision fell outside the exact glibc-exp table (never seen) */
};

/* Boundary conditions along z (PROGRAM/Makefile:8-30, ini.c:551-641). */
enum { EA_PBC = 0, EA_OBC = 1, EA_OBC_WEAK = 2, EA_OBC_STRONG = 3 };

typedef struct {
  int32_t L, Lz;     /* multiples of 8 (header.h:41-47) */
  int32_t nbetas;    /* NBETAS, 2..255 */
  int32_t nrep;      /* NR, 8 in the reference (header.h:14); the Houdayer move needs NR/2 >= 2 */
  int32_t nsamples;  /* nbits, 1..32 (main.cu:53) */
  int32_t bc;        /* EA_PBC / EA_OBC / EA_OBC_WEAK / EA_OBC_STRONG */
} ea_geom;

/* Host generator states, byte-compatible with the reference's structs
 * (PROGRAM/include/random_generator.h:31-46) and its checkpoint files. */
typedef struct {
  uint64_t ira[256];
  uint64_t PR, zseed, final;
  uint8_t ip, ip1, ip2, ip3;
  uint8_t padding[4];
} ea_hq;
typedef struct {
  uint64_t s[4];
  uint64_t t, final;
} ea_xoshiro;

/* All generator state of a job (Init_Random, PROGRAM/src/ini.c:61-101). */
typedef struct {
  ea_hq prc[64];            /* Parisi-Rapuano per replica, feeds the Philox counters */
  ea_xoshiro xo[64];        /* xoshiro256++ per replica */
  uint32_t keys[64];        /* Philox key word per replica */
  ea_hq rc;                 /* random_c: Houdayer replica choice */
  uint64_t cuda_rng_offset; /* uniforms consumed by the cluster moves so far */
  uint64_t seed_cluster;    /* cuRAND XORWOW seed */
} ea_generators;

/* Cadence of one bin (input file fields, PROGRAM/src/io.c:399-436). */
typedef struct {
  int32_t itmax, houfr, mesfr, ptfr;
  int32_t cluster;   /* 0 = NO_CLUSTER build of the reference */
  int32_t nclust;    /* beta indices (coldest first) in the Houdayer move; <=0: lround(0.5*NB) */
} ea_cadence;

const char *ea_last_error(void);
int ea_version(void);
/* Number of visible CUDA devices (cudaGetDeviceCount, main.cu:64). */
int ea_device_count(int32_t *count);

/* ---- host-side set-up (no GPU involved) -------------------------------------
 * Seeds, couplings and initial spins exactly as the reference builds them. */

/* generate_seed_vectors + Init_Random (ini.c:32-101): per-sample seeds_J/seeds_u,
 * per-replica seeds_MC, and every generator state.  list_samples may be NULL
 * (0..nsamples-1).  pt_out: [nsamples][NR] states of the PT generators. */
int ea_host_seeds(uint64_t master_J, uint64_t master_u, uint64_t master_MC, uint64_t master_cluster,
                  const int32_t *list_samples, int32_t nsamples, int32_t nrep,
                  uint64_t *seeds_J, uint64_t *seeds_u, uint64_t *seeds_MC);
int ea_host_generators(const uint64_t *seeds_MC, const int32_t *list_samples, int32_t nsamples,
                       int32_t nrep, uint64_t seed_cluster, ea_generators *gen, ea_hq *pt_out);
/* Init_u + packing_u (ini.c:316-383). even/odd: [NB][half][NR]. */
int ea_host_init_spins(const ea_geom *g, uint64_t seed_u, uint64_t *even, uint64_t *odd);
/* Init_J + packing_J (ini.c:465-730).  J6 (may be NULL): the six V-byte planes
 * Jx,Jy,Jz,Jmx,Jmy,Jmz written to couplings.bin (io.c:284-305).  Jw: [2][6][half]. */
int ea_host_init_couplings(const ea_geom *g, uint64_t seed_J, uint8_t *J6, uint64_t *Jw, int32_t *countJ);
/* unpacking_u / packing_u for one replica: spins of every clone as bytes [NB][V] in
 * natural site order x + L*y + L*L*z (ini.c:385-433). */
int ea_host_unpack_replica(const ea_geom *g, const uint64_t *even, const uint64_t *odd, int32_t rep, uint8_t *u);
int ea_host_pack_replica(const ea_geom *g, const uint8_t *u, int32_t rep, uint64_t *even, uint64_t *odd);
/* calculate_scalar_energy (med.c:3-44) of one clone given as V bytes. */
int ea_host_scalar_energy(const ea_geom *g, const uint8_t *u, const uint8_t *J6, int32_t *E);

/* ---- device context ------------------------------------------------------------ */
typedef struct ea_ctx ea_ctx;

/* Allocates the job on `device` (cudaSetDevice + cudaMalloc once, here). */
int ea_create(const ea_geom *g, int32_t device, ea_ctx **out);
int ea_destroy(ea_ctx *ctx);
int ea_get_geom(const ea_ctx *ctx, ea_geom *g);
/* Waits for all work of the context (its stream and its generator stream). */
int ea_sync(ea_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), so callers can order their own
 * work or timing events with the job's kernels.  The cluster uniforms of the
 * next Houdayer move are drawn ahead on a second stream of the context. */
int ea_get_stream(ea_ctx *ctx, void **stream);
/* Makes the context's stream wait for the work queued so far on its
 * generator stream (the uniforms drawn ahead), without a host
 * synchronisation: an event recorded on the stream afterwards covers all
 * work of the job.  No reference counterpart (the reference draws the
 * uniforms inside the move, HoudayerXEA.cu:189-195). */
int ea_join(ea_ctx *ctx);

/* Inputs.  betas descending (read_betas, io.c:476-501); cum: [NB][256] (read_lut, io.c:504-534). */
int ea_set_temperatures(ea_ctx *ctx, const double *betas, const uint64_t *cum);
int ea_set_spins(ea_ctx *ctx, int32_t sample, const uint64_t *even, const uint64_t *odd);
int ea_get_spins(ea_ctx *ctx, int32_t sample, uint64_t *even, uint64_t *odd);
/* The spins of every sample, [nsamples][2][NB][half][NR] (each sample's even
 * then odd array, as ea_set_spins takes them), in one copy enqueued on the
 * context's stream without a host synchronisation: the buffer should be
 * pinned (cudaHostAlloc) and stay unchanged until the stream has passed the
 * copy (ea_sync, or a later call that returns data).  No reference
 * counterpart (the reference uploads at start-up and restarts only). */
int ea_upload_spins_async(ea_ctx *ctx, const uint64_t *all);
/* The two halves of ea_upload_spins_async, so that the host copy of the next
 * state can run beside the current kernels: ea_stage_spins_async starts the
 * host-to-device copy of a whole state (layout as above) into a staging
 * buffer of the context (allocated at the first call, the size of the spins)
 * on a copy stream of its own, without touching the job's spins;
 * ea_commit_staged_spins makes the context's stream wait for that copy and
 * move the staged state into the spins (a device copy).  The host buffer
 * must stay unchanged until the commit has been passed by the stream. */
int ea_stage_spins_async(ea_ctx *ctx, const uint64_t *all);
int ea_commit_staged_spins(ea_ctx *ctx);
int ea_set_couplings(ea_ctx *ctx, int32_t sample, const uint64_t *Jw);
/* pt: [nsamples][NR] PT generators (random_PT, header.h:133). */
int ea_set_generators(ea_ctx *ctx, const ea_generators *gen, const ea_hq *pt);
int ea_get_generators(ea_ctx *ctx, ea_generators *gen, ea_hq *pt);
/* which_clon_this_beta [nsamples][NR][NB]; NULL = identity (init_tempering, ini.c:763-781). */
int ea_set_permutations(ea_ctx *ctx, const uint8_t *wctb);
int ea_get_permutations(ea_ctx *ctx, uint8_t *wctb, uint8_t *wbtc);
/* PT acceptance accumulators [nsamples][NR][NB-1] (aceptancePT, attemptsPT, aceptancePTraw). */
int ea_get_pt_stats(ea_ctx *ctx, double *acc, double *att, double *accraw);
int ea_reset_pt_stats(ea_ctx *ctx);
/* Philox time counter and 14-bit job id (main.cu:59-62,139; fill_bits.h:47-68). */
int ea_set_counter(ea_ctx *ctx, int64_t iter, uint32_t jobid);
int ea_get_counter(ea_ctx *ctx, int64_t *iter);

/* ---- the hot path ------------------------------------------------------------------ */
/* Monte_Carlo (main.cu:285-349): nsweeps x {even, odd} half-sweeps of the fused
 * heat-bath-LUT + Metropolis kernel.  The energies of the final state are
 * accumulated inside the last odd half-sweep (consumed by ea_parallel_tempering). */
int ea_monte_carlo(ea_ctx *ctx, int32_t nsweeps);
/* Measure_Energy (main.cu:531-554).  out may be NULL (result stays on the device). */
int ea_measure_energy(ea_ctx *ctx, int32_t *out);
/* Energy measurement that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc -- frameworks that hand
 * out every device byte from their own pool (a cudaMalloc behind their back
 * breaks their accounting and can fail when the pool holds the memory), and
 * loops that cannot take the device-wide synchronisation an allocation may
 * imply.  Same result as ea_measure_energy for
 * spins [nsamples][2][NB][half][NR] and couplings [nsamples][2][6][half]
 * already in device memory; writes energies [nsamples][NR][NB] (int32) to
 * d_energies on `stream` (a cudaStream_t, NULL = legacy default stream), on
 * the calling thread's current device.  NR must be 2, 4 or 8 (the tile
 * widths KT = 16, 8, 4 of the energy kernel); other replica counts get
 * EA_ERR_ARG.  Its scratch is a fixed 4.4 MiB device array inside the
 * library (held by every GPU that loads it until exit), so it rejects, with
 * EA_ERR_ARG and a message, jobs beyond
 * (L/4)^2 (Lz/4) / 2 <= 8192 half-sites and
 * ceil(half/KT) * nsamples * NB * NR <= 2^20 partial sums (KT = 32/NR).
 * The first call on each device (and the first after that device's context
 * is recreated, e.g. by cudaDeviceReset) looks up the array's device address;
 * make that first call before any stream capture.  All calls share the array,
 * so calls whose kernels overlap on the GPU race; serialise them (one stream,
 * or events).  Nothing in the array needs to start at zero.  A CUDA error
 * already pending on the calling thread when it is called is reported (and
 * left pending) instead of being taken for a failure of this call. */
int ea_measure_energy_noalloc(const ea_geom *g, const uint64_t *d_spins, const uint64_t *d_couplings,
                              int32_t *d_energies, void *stream);
/* Parallel_Tempering for every (sample, replica) (upd.c:3-48) on the device, with
 * the reference's FP64 arithmetic and glibc exp() values tabulated on the host. */
int ea_parallel_tempering(ea_ctx *ctx);
/* Houdayer (main.cu:351-453 + HoudayerXEA.cu): two replica groups, cuRAND XORWOW
 * uniforms with the reference's seed/offset/sizes, min-index cluster roots. */
int ea_houdayer(ea_ctx *ctx, int32_t nclust);
/* Bond rule of the cluster labelling.  EA_CLUSTER_REFERENCE (default)
 * reproduces the reference binary: site 0 tests its periodic -x bond against
 * x = (2^32-1+L) mod L (a 32-bit wrap in HoudayerXEA.cu:96) while still joining
 * sites 0 and L-1; it equals the correct rule when L is a power of two.
 * EA_CLUSTER_EXACT tests the bond against x = L-1, so every move conserves
 * E(r1)+E(r2) for every L. */
enum { EA_CLUSTER_REFERENCE = 0, EA_CLUSTER_EXACT = 1 };
int ea_set_cluster_rule(ea_ctx *ctx, int32_t rule);
/* SM split between the cluster-uniform generator and the job's kernels.
 * cuRAND's XORWOW generator runs 64 blocks of 64 threads whose length is set
 * by the call size; on its own green-context partition of nsm SMs it keeps
 * its full speed (nsm >= 32) while the job's kernels run on the other SMs,
 * and the two overlap.  nsm = 0: no partition (the generator runs on a
 * high-priority stream over the whole device); nsm < 0: automatic, 32 SMs when
 * a move draws at least 2^24 uniforms (ea_create applies it), else none.
 * Allowed before the first cluster move only; it replaces the context's
 * streams, so a handle from ea_get_stream taken earlier is stale.  No
 * reference counterpart (results do not depend on it). */
int ea_set_rng_sms(ea_ctx *ctx, int32_t nsm);
/* SMs of the generator's partition (0: none). */
int ea_get_rng_sms(const ea_ctx *ctx, int32_t *nsm);
/* One bin (main.cu:149-230): itmax x mesfr x (houfr x (MC + energy + PT) + Houdayer),
 * then the per-it energy measure, average and temperature-history record.
 * avgE [nsamples][NR][NB] (sum over it, beta order) and hist [nsamples][NR][maxit][NB]
 * may be NULL; maxit_trw = itmax / frecTRW (io.c:431-434). */
int ea_run_bin(ea_ctx *ctx, const ea_cadence *cad, double *avgE, uint8_t *hist, int32_t *maxit_trw);
/* Energy averages, temperature history and maxit_trw of the job's last bin
 * (by ea_run_bin or a batch), as ea_run_bin returns them. */
int ea_bin_results(ea_ctx *ctx, double *avgE, uint8_t *hist, int32_t *maxit_trw);

/* Batches.  A batch advances many jobs -- of different L, Lz, boundary
 * condition, number of temperatures and samples, same number of replicas and
 * device -- with one persistent kernel launch per step for all of them (a
 * packed work list of (job, block) items); the sweep / energy / tempering
 * cycle is replayed as a CUDA graph.  Each job's words, energies, swaps and
 * uniforms are those of ea_run_bin on the job alone.  The batch fixes the
 * jobs' sweep tile width (tile = 0: chosen from the work list; else 1, 2, 4,
 * 8 or 16 as the replica count allows).  A job's own calls may be used
 * between batch calls; they are ordered after the batch.  No reference
 * counterpart: the reference runs one job per process. */
typedef struct ea_batch ea_batch;
int ea_batch_create(ea_ctx *const *jobs, int32_t njobs, int32_t tile, ea_batch **out);
int ea_batch_destroy(ea_batch *b);
int ea_batch_tile(const ea_batch *b, int32_t *tile);
/* Replaces the batch's jobs between bins (continuous batching): jobs that
 * stay keep their state, new ones join with the batch's tile width, jobs that
 * leave are ordered after the bins they took part in.  The new work list is
 * uploaded in stream order, so the call does not wait for bins in flight.
 * Fails with EA_ERR_ARG if the largest NB no longer fits the tile width. */
int ea_batch_set_jobs(ea_batch *b, ea_ctx *const *jobs, int32_t njobs);
/* One bin of the cadence for every job, enqueued without a host
 * synchronisation; read each job's results with ea_bin_results. */
int ea_batch_run_bin(ea_batch *b, const ea_cadence *cad);
int ea_batch_sync(ea_batch *b);
/* The batch's CUDA stream (a cudaStream_t). */
int ea_batch_stream(ea_batch *b, void **stream);
/* With avgE and hist both NULL, ea_run_bin only enqueues the bin and returns
 * without synchronising; ea_check_exact then synchronises and reports
 * EA_ERR_INEXACT if any tempering decision fell outside the exact exp table. */
int ea_check_exact(ea_ctx *ctx);

/* Per-kernel timing: while enabled, every launch of the listed kernels is
 * bracketed by CUDA events on the context's stream.  ea_kernel_time syncs and
 * returns the number of launches and their summed duration since enabling. */
enum { EA_K_SWEEP = 0, EA_K_PT = 1, EA_K_CLUSTER = 2, EA_K_ENERGY = 3, EA_K_RNG = 4, EA_K_COUNT = 5 };
int ea_profile(ea_ctx *ctx, int32_t on);
int ea_kernel_time(ea_ctx *ctx, int32_t kind, int64_t *launches, double *total_ms);
/* Measured peak rate of 32-bit integer instructions on a device, in thread
 * operations per second over all SMs: independent xor/add chains
 * (alu_ops_per_s) and multiply-add chains (imad_ops_per_s; either pointer
 * may be NULL).  No counterpart in the reference: it is the denominator of
 * the integer-pipe roofline of the sweep kernels. */
int ea_probe_int32_rate(int32_t device, double *alu_ops_per_s, double *imad_ops_per_s);

/* A new run (flag 1 of the reference) on an existing context, as Init() does
 * (ini.c:32-101, 316-383, 465-730, 763-781): seeds from the four master seeds
 * (seed_J, seed_u, seed_MC, seed_cluster), generators, initial spins,
 * couplings, identity permutations, then the Philox counter and job id
 * (main.cu:59-62).  list_samples may be NULL (samples 0..nsamples-1). */
int ea_init_run(ea_ctx *ctx, const uint64_t masters[4], const int32_t *list_samples, int64_t iter0, uint32_t jobid);
/* Upper bound of the device bytes a job of geometry g holds once it has run
 * bins of cadence cad (NULL: no bin yet) -- what admission by an HBM budget
 * charges for it.  betas (may be NULL) sizes the tempering exp table exactly. */
int ea_job_bytes(const ea_geom *g, const ea_cadence *cad, const double *betas, uint64_t *bytes);

/* ---- sample-packed layout: any L >= 2, Lz >= 2, any number of replicas -------
 * No reference counterpart: the reference's multispin words hold 64 spatial
 * sub-blocks of one sample, so L and Lz must be multiples of 8
 * (header.h:41-47).  Here a word holds the same site of 64 disorder samples
 * (bit b = sample b), so a job of `nwords` words simulates 64*nwords samples
 * of any L x L x Lz tube.  The dynamics are the reference's, per sample: the
 * Philox + heat-bath-threshold random words shared by all samples
 * (main.cu:994-1150), the bit-sliced Metropolis rule (main.cu:1474-1506), six
 * bond slots per site with the reference's fake bond on open z planes
 * (ini.c:551-641; for odd L, see ea_sp_graph), E = 3V - 2 x unsatisfied bonds,
 * and the tempering rule of upd.c:3-48 per (sample, replica) chain with a
 * counter-based uniform.  Sites are updated colour by colour (a proper
 * colouring of the bond graph: 2 colours when the tube is bipartite, else
 * 3 or more).  Temperature slots keep their beta; accepted swaps move the
 * samples' configurations between slots.
 *
 * Layouts: spins [nwords][V][NR][NB] (slot-major last), couplings
 * [nwords][V][6] (slots +x,+y,+z,-x,-y,-z; both ends of a bond hold the same
 * word), energies and permutations [nwords][64][NR][NB], site = x + L*(y + L*z). */
typedef struct {
  int32_t L, Lz, nbetas, nrep, nwords, bc;  /* bc: EA_PBC or EA_OBC; nbetas <= 64 */
} ea_sp_geom;
typedef struct ea_sp ea_sp;

/* Bond graph (host only): nb [V][6] neighbour of each slot, mate [V][6] the
 * half-edge p*6+slot at the other end, colour [V], ncol.  Any pointer may be
 * NULL.  Open z planes: the missing z slot holds a fake bond; for even L to
 * the y neighbour chosen by the parity of x+y+z (as the reference pairs
 * them); for odd L to x+-1 (x < L-1), else y+-1 (y < L-1), and site
 * (L-1, L-1) pairs with the same site of the other open plane. */
int ea_sp_graph(int32_t L, int32_t Lz, int32_t bc, int32_t *nb, int32_t *mate, uint8_t *colour, int32_t *ncol);
/* Couplings and initial spins as ea_sp_init makes them (host only). */
int ea_sp_host_init(const ea_sp_geom *g, uint64_t seed_J, uint64_t seed_u, uint64_t *J, uint64_t *S);
/* The 11-bit pre-search table of one temperature's 256 thresholds, as the
 * per-item colour pass stages it (host only; no reference counterpart):
 * pre[t] = the first byte n with (t << 53) < cum[n] for t < 2048, and 255
 * for t = 2048..2063.  The byte of a key R lies in [pre[R >> 53],
 * pre[(R >> 53) + 1]].  cum[255] must be 2^64-1. */
int ea_sp_presearch11(const uint64_t *cum, uint8_t *pre);
int ea_sp_create(const ea_sp_geom *g, int32_t device, ea_sp **out);
int ea_sp_destroy(ea_sp *job);
int ea_sp_info(const ea_sp *job, int32_t *ncol, int32_t *tile);
int ea_sp_stream(ea_sp *job, void **stream);
int ea_sp_sync(ea_sp *job);
int ea_sp_set_temperatures(ea_sp *job, const double *betas, const uint64_t *cum);
/* seeds: seed_J, seed_u, seed_MC (Metropolis generators per replica, as
 * Init_Random seeds them), seed_PT (tempering uniforms). */
int ea_sp_init(ea_sp *job, const uint64_t seeds[4], uint32_t jobid);
int ea_sp_set_generators(ea_sp *job, const ea_generators *gen, uint64_t pt_seed);
int ea_sp_get_generators(ea_sp *job, ea_generators *gen);
int ea_sp_set_spins(ea_sp *job, const uint64_t *S);
int ea_sp_get_spins(ea_sp *job, uint64_t *S);
int ea_sp_set_couplings(ea_sp *job, const uint64_t *J);
/* Colour-pass counter (Philox time) and tempering step counter. */
int ea_sp_set_counter(ea_sp *job, int64_t iter, uint64_t ptstep, uint32_t jobid);
int ea_sp_get_counter(ea_sp *job, int64_t *iter, uint64_t *ptstep);
/* n Metropolis sweeps (every colour pass). */
int ea_sp_sweeps(ea_sp *job, int32_t n);
/* Unsatisfied half-edges U2 [nwords][64][NR][NB] (E = 3V - U2); NULL: on the device only. */
int ea_sp_energy(ea_sp *job, int32_t *U2);
/* Energies, then one tempering step for every chain, then the swaps applied to the spins. */
int ea_sp_parallel_tempering(ea_sp *job);
/* E and perm [nwords][64][NR][NB] after the last step, accepted swaps
 * [nwords][64][NR][NB-1], lane masks of the last step [nwords][NR][NB-1]. */
int ea_sp_get_tempering(ea_sp *job, int32_t *E, uint8_t *perm, uint32_t *acc, uint64_t *masks);
/* Houdayer move (main.cu:351-453) per sample, on the nclust coldest slots
 * (<= 0: lround(NB/2)): replica pairs from random_c as the reference picks
 * them (two groups of NR/2, one group when NR < 4), maximal clusters of equal
 * overlap along all six bond slots (fake bonds included: E(r1)+E(r2) is
 * conserved for any L), smallest-site roots, each cluster flipped in both
 * replicas with probability 1/2 (a Philox bit of move, root, sample, slot,
 * group).  Lattices up to 32768 sites are labelled in shared memory, larger
 * ones in a device scratch area of 7 bytes per site and labelled lattice. */
int ea_sp_houdayer(ea_sp *job, int32_t nclust);
/* One bin of the reference's cadence (main.cu:149-230): itmax x [mesfr x
 * (houfr x (ptfr sweeps + tempering) + Houdayer if cad->cluster) + energy
 * measurement]; avgE [nwords][64][NR][NB] (may be NULL) = the bin's average
 * energy of each slot. */
int ea_sp_run(ea_sp *job, const ea_cadence *cad, double *avgE);
/* The last bin's average energies (by ea_sp_run or a batch), as ea_sp_run returns them. */
int ea_sp_bin_results(ea_sp *job, double *avgE);
/* How ea_sp_run (and ea_sp_batch_run) executes a bin.  EA_BIN_GRAPH: one
 * bin iteration replayed as a CUDA graph of one launch per phase (colour
 * pass, energy, tempering, permute, labelling, ...).  EA_BIN_PERSISTENT: one
 * cooperative launch of a persistent kernel runs the whole bin, the same
 * phase bodies in the same order separated by grid barriers, so the results
 * are identical; it removes the per-phase launch gaps that bound jobs too
 * small to fill the GPU.  A barrier wait gives up after 4 s (the kernel
 * returns) and the next ea_sp_sync / ea_sp_bin_results / ea_sp_batch_sync
 * reports EA_ERR_CUDA.  EA_BIN_RESIDENT (jobs alone whose words fit in one
 * thread-block cluster of up to 16 CTAs): per launch of up to 16 MB of
 * random words, the Philox counters of every colour pass, then all random
 * words on the whole GPU, then one cluster keeps the spin and coupling
 * words in its distributed shared memory and runs every sweep, energy
 * count, tempering step and measurement, with the same results; with
 * cluster moves every block of houfr x ptfr >= 4 sweeps is one such launch
 * and the moves run as per-phase launches between them; other bins get
 * EA_ERR_ARG.  EA_BIN_AUTO (default): the
 * resident kernel where it applies, else the graph (the persistent kernel
 * measured slower than the graph for a small job alone and for batches of
 * small jobs: a batch's phases in lock-step wait for each phase's slowest
 * job).  Batches take AUTO, GRAPH or PERSISTENT. */
enum { EA_BIN_AUTO = 0, EA_BIN_GRAPH = 1, EA_BIN_PERSISTENT = 2, EA_BIN_RESIDENT = 3 };
int ea_sp_set_bin_kernel(ea_sp *job, int32_t mode);
/* The form (EA_BIN_GRAPH, EA_BIN_PERSISTENT or EA_BIN_RESIDENT) ea_sp_run
 * takes for a bin of this cadence. */
int ea_sp_bin_kernel_for(ea_sp *job, const ea_cadence *cad, int32_t *mode);
/* Autotuner (no reference counterpart): times, on the job itself, the launch
 * shapes that leave every result unchanged -- the colour pass's form (tiles
 * of `tile` sites staging their random words in SMEM, or tile 0: the
 * per-item pass, one thread per (site, replica, slot) drawing its own words
 * on a grid of resident CTAs), the energy count's sites per thread and the
 * cluster labelling's block size -- and keeps the fastest of each; the job's
 * state is saved on the device and put back, so its results are those of the
 * untuned job.  Allocates the overlap buffer of the cluster moves if it is
 * missing.  Outputs may be NULL. */
int ea_sp_autotune(ea_sp *job, int32_t *tile, int32_t *echunk, int32_t *cthreads);
/* Sets the colour pass's form by hand: tile > 0 sites per CTA (1..64, the
 * CTA's tables fitting in SMEM), or 0 for the per-item pass.  The words are
 * the same in every form.  A job starts with the per-item pass if it has one
 * sample word, else with tiles of a heuristic width; batches run each job's
 * form.  ea_sp_info reports the form in force. */
int ea_sp_set_tile(ea_sp *job, int32_t tile);
/* Configuration analysis of the job's current spins (no reference code; the
 * reference's DATA/README.md describes correlation functions of the overlap
 * built from f, g in {x, x^3, sign x} with r = 2, 4, 6, 8 replicas).  The
 * replica pairs are (0,1), (2,3), ... among the first nrep replicas (even,
 * <= NR); the plane overlap of a pair at a temperature slot and plane z is
 * q_z = 1 - 2 diff_z / L^2, diff_z = spins that differ on the plane (planes
 * of at most 4095 sites).
 * ea_sp_plane_overlaps: diff [nwords][64][nrep/2][NB][Lz].
 * ea_sp_plane_correlations: C [nwords*64][NB][dmax+1][3][3], entry [f][g] =
 * mean over the pairs and planes z of f(q_z) g(q_{z+d}) for f, g in
 * (x, x^3, sign x); z + d taken modulo Lz under PBC, only z + d < Lz with
 * open boundaries; dmax < Lz. */
int ea_sp_plane_overlaps(ea_sp *job, int32_t nrep, int32_t *diff);
int ea_sp_plane_correlations(ea_sp *job, int32_t nrep, int32_t dmax, double *C);
/* Batches of sample-packed jobs (any geometries, replica and temperature
 * counts, up to 4 colours each).  Jobs are grouped in classes (one per job
 * for up to 256 jobs, else of equal NB and similar lattice size); each class
 * takes one launch per kernel kind over a packed (job, block) work list,
 * sized for the class, and one bin iteration of all classes -- side by side,
 * one graph branch each -- is replayed as one CUDA graph launch.  Each job's words, energies and swaps equal those of
 * ea_sp_run on the job alone.  Asynchronous; read results with
 * ea_sp_bin_results. */
typedef struct ea_sp_batch ea_sp_batch;
int ea_sp_batch_create(ea_sp *const *jobs, int32_t njobs, ea_sp_batch **out);
int ea_sp_batch_run(ea_sp_batch *b, const ea_cadence *cad);
int ea_sp_batch_sync(ea_sp_batch *b);
int ea_sp_batch_stream(ea_sp_batch *b, void **stream);
int ea_sp_batch_destroy(ea_sp_batch *b);
/* EA_BIN_* for the batch's bins (see ea_sp_set_bin_kernel). */
int ea_sp_batch_set_bin_kernel(ea_sp_batch *b, int32_t mode);
/* Exact enumeration (V <= 32): dos [nwords*64][6V+1] configurations with
 * spin 0 up at each E = -3V..3V, and meanE [nwords*64][nbeta] = <E>(beta)
 * from it in FP64 on the GPU. */
int ea_sp_exact(ea_sp *job, const double *betas, int32_t nbeta, uint64_t *dos, double *meanE);
/* Upper bound of the device bytes of a sample-packed job after bins of cadence cad (NULL: none). */
int ea_sp_job_bytes(const ea_sp_geom *g, const ea_cadence *cad, const double *betas, uint64_t *bytes);

/* ---- serving: continuous batching of simulation jobs -------------------------
 * A server owns one device and a worker thread.  Submitted jobs wait in a
 * queue until their device bytes (ea_job_bytes) fit the HBM budget and a slot
 * is free; admitted jobs are created and initialised as new runs
 * (ea_init_run), join the batch of their replica count and cadence, and are
 * advanced one bin per step by the batched kernels, interleaved with every
 * other running job; a job leaves its batch after its last bin.  Up to
 * `depth` bins per batch are in flight, and the job list of a batch changes
 * between bins without draining the GPU.  Each job's words, energies, swaps
 * and uniforms equal those of the same job run alone by ea_run_bin.  Latency
 * is submission to completion as the worker observes it (host clock).  A
 * finished job's context stays readable (ea_get_spins, ea_bin_results, ...)
 * until ea_server_release.  No reference counterpart: the reference runs one
 * job per process. */
typedef struct ea_server ea_server;
typedef struct {
  int32_t device;
  int32_t max_jobs;      /* jobs admitted at once (<= 0: 1024) */
  int32_t depth;         /* bins in flight per batch (<= 0: 2) */
  int32_t tile;          /* sweep tile width of the batches (0: the widest that fits nb_max) */
  int32_t nb_max;        /* largest accepted NB (<= 0: 64) */
  int32_t reserved;
  uint64_t hbm_budget;   /* device bytes the jobs may hold (0: 90 % of the free memory at creation) */
} ea_server_config;

enum { EA_LAYOUT_MULTISPIN = 0, EA_LAYOUT_SAMPLE_PACKED = 1 };
typedef struct {
  ea_geom geom;          /* sample-packed: nsamples unused, see nwords */
  const double *betas;   /* [nbetas], copied */
  const uint64_t *cum;   /* [nbetas][256], copied */
  uint64_t masters[4];   /* multispin: seed_J, seed_u, seed_MC, seed_cluster; sample-packed: ea_sp_init's seeds */
  ea_cadence cad;        /* one bin */
  int32_t nbins;         /* bins to run (>= 1) */
  uint32_t jobid;        /* 14-bit Philox job id */
  int64_t iter0;         /* initial half-sweep counter (multispin) */
  int32_t layout;        /* EA_LAYOUT_MULTISPIN: batched with its class; EA_LAYOUT_SAMPLE_PACKED:
                            any L, Lz >= 2, bins on the job's own stream */
  int32_t nwords;        /* sample-packed: words of 64 samples */
} ea_request;

enum { EA_JOB_QUEUED = 0, EA_JOB_RUNNING = 1, EA_JOB_DONE = 2, EA_JOB_FAILED = 3, EA_JOB_RELEASED = 4 };
typedef struct {
  int32_t state;
  int32_t bins_done;
  double t_submit, t_admit, t_done;  /* seconds since the server's creation (-1: not yet) */
  uint64_t bytes;                    /* charged against the budget */
  double spin_updates;
  double t_ready;   /* created and initialised by a preparation thread */
  double t_start;   /* its first bin enqueued */
  double gpu_s;     /* device time of the bins it took part in (a batch's bin counts for each member) */
} ea_job_info;

typedef struct {
  int64_t submitted, admitted, completed, failed, queued, running;
  int64_t bins, batch_changes, peak_running;
  double p50_ms, p99_ms, mean_ms, max_ms;  /* completion latency of the completed jobs */
  double spin_updates;                     /* of the completed jobs */
  double span_s;                           /* first submission to last completion */
  uint64_t budget, bytes_in_use, bytes_peak;
  double gpu_busy_s;  /* sum of the bins' device durations (CUDA events) */
  double enqueue_s;   /* worker time spent enqueueing bins (batch changes included) */
  double admit_s;     /* worker time spent creating and initialising admitted jobs */
  /* Components of the completed jobs' latency, p50 / p99 in ms: queue wait
   * (submission to admission by the HBM budget and the slots), preparation
   * (admission to created and initialised), start wait (to the first bin
   * enqueued) and run (first bin to completion); and the jobs' bin device
   * time. */
  double queue_p50_ms, queue_p99_ms, prep_p50_ms, prep_p99_ms, start_p50_ms, start_p99_ms;
  double run_p50_ms, run_p99_ms, gpu_p50_ms, gpu_p99_ms;
} ea_serve_stats;

int ea_server_create(const ea_server_config *cfg, ea_server **out);
/* Queues a job; returns EA_ERR_ARG for a request that can never run (bad
 * geometry, NB above nb_max, bytes above the budget). */
int ea_server_submit(ea_server *s, const ea_request *r, int64_t *ticket);
/* Waits until the job is done or failed (timeout_s < 0: no limit); job (may be
 * NULL) receives its context, still owned by the server.  EA_ERR_STATE on
 * timeout; the job's own error code if it failed. */
int ea_server_wait(ea_server *s, int64_t ticket, double timeout_s, ea_ctx **job);
int ea_server_info(ea_server *s, int64_t ticket, ea_job_info *info);
/* The sample-packed job of a finished request (ea_server_wait's job is NULL for those). */
int ea_server_sp_job(ea_server *s, int64_t ticket, ea_sp **job);
/* Frees a finished job's device memory (asynchronously; the budget is
 * credited once it is freed). */
int ea_server_release(ea_server *s, int64_t ticket);
int ea_server_stats(ea_server *s, ea_serve_stats *st);
/* Waits until every submitted job has finished. */
int ea_server_drain(ea_server *s);
/* Cancels queued jobs, waits for the running ones' bins and frees everything. */
int ea_server_destroy(ea_server *s);


/* cuRAND XORWOW uniforms (device generator) for a seed/offset, copied to host.
 * Used to check the device generator against the host one. */
int ea_curand_uniforms(int32_t device, uint64_t seed, uint64_t offset, uint64_t n, double *out);

#ifdef __cplusplus
}
#endif
#endif
