// api.cu -- the C ABI of libeagb.so (declared in include/eagb.h).
//
// A context is one job: it owns every device buffer and two streams (the job's
// and the cluster-uniform generator's), and enqueues the kernels of kernels.cu
// in the order of the reference driver (PROGRAM/src/main.cu:142-230).  No call
// synchronises the device except the ones that return data to the host.
#include <cuda.h>
#include <curand.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "eagb.h"
#include "host.hpp"
#include "batch.cuh"
#include "kernels.cuh"

using namespace eagb;

namespace {
thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CU(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return fail(EA_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));     \
  } while (0)

#define CR(call)                                                                                  \
  do {                                                                                            \
    curandStatus_t e_ = (call);                                                                   \
    if (e_ != CURAND_STATUS_SUCCESS) return fail(EA_ERR_CURAND, "%s: curand status %d", #call, (int)e_); \
  } while (0)

template <class T>
cudaError_t dalloc(T *&p, size_t n) {
  return cudaMalloc((void **)&p, sizeof(T) * (n ? n : 1));
}
}  // namespace

struct ea_ctx {
  Geometry g;
  int device = 0;
  cudaStream_t st = nullptr;
  JobDev j{};
  std::vector<void *> owned;
  bool have_temps = false;
  bool energies_fresh = false;
  // Houdayer
  curandGenerator_t gen = nullptr;
  uint64_t cuda_rng_offset = 0, seed_cluster = 0;
  int nclust_cap = 0;
  // Uniforms of a move: U[set][group].  The generator runs on its own stream
  // `rs` at the highest priority and draws the next move's set while the
  // current move and the sweeps after it run on `st`.  Its kernel holds 64
  // blocks of 64 threads and is bound by FP64 throughput on the SMs it
  // holds, so it overlaps the integer kernels of the job almost entirely.
  // The sequence of uniforms is the generator's own, whatever the overlap.
  cudaStream_t rs = nullptr;
  // optional SM partition (green contexts): the generator on its own SMs,
  // the job's kernels on the rest
  CUgreenCtx part[2] = {nullptr, nullptr};
  int part_sms = 0;
  double *U[2][2] = {};
  cudaEvent_t drawn[2] = {}, used[2] = {};
  int cur = 0;    // set that holds the uniforms of the next move
  int ready = 0;  // sets drawn and not yet used by a move (0..2)
  uint32_t *label = nullptr;
  uint32_t *sel = nullptr;
  unsigned long long *Q = nullptr;
  // measurement buffers
  double *avgE = nullptr;
  uint8_t *hist = nullptr;
  int hist_cap = 0;
  std::vector<int32_t> expoff;
  double *exptab = nullptr;
  // staging of whole spin states uploaded from the host (ea_stage_spins_async):
  // the host copy runs on `cs` into `stage`, beside the job's kernels
  cudaStream_t cs = nullptr;
  unsigned long long *stage = nullptr;
  cudaEvent_t staged = nullptr, stage_free = nullptr;
  bool stage_pending = false;
  // per-kernel timing (ea_profile)
  bool prof_on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_ev[EA_K_COUNT];
  int64_t prof_n[EA_K_COUNT] = {};
  double prof_ms[EA_K_COUNT] = {};
};

namespace {

template <class T>
int own(ea_ctx *c, T *&p, size_t n) {
  cudaError_t e = dalloc(p, n);
  if (e != cudaSuccess) return fail(EA_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", sizeof(T) * n, cudaGetErrorString(e));
  c->owned.push_back((void *)p);
  cudaMemsetAsync(p, 0, sizeof(T) * (n ? n : 1), c->st);
  return EA_OK;
}

int choose_kt(const Geometry &g) {
  const char *env = getenv("EAGB_KT");
  auto smem = [&](int kt) { return sweep_smem_for(g.NB, g.NR, kt); };
  const int cands_nr8[3] = {4, 2, 1}, cands_nr4[3] = {8, 4, 2}, cands_nr2[3] = {16, 8, 4};
  const int *c = g.NR == 8 ? cands_nr8 : g.NR == 4 ? cands_nr4 : cands_nr2;
  if (env) {
    int kt = atoi(env);
    for (int i = 0; i < 3; ++i)
      if (c[i] == kt && smem(kt) <= 227 * 1024) return kt;
  }
  for (int i = 0; i < 3; ++i) {
    const int kt = c[i];
    const int tiles = (g.half + kt - 1) / kt;
    if (smem(kt) <= 227 * 1024 && tiles >= 2 * 152) return kt;
  }
  for (int i = 2; i >= 0; --i)
    if (smem(c[i]) <= 227 * 1024) return c[i];
  return 0;
}

int check(ea_ctx *c) {
  if (!c) return fail(EA_ERR_ARG, "null context");
  return EA_OK;
}

int set_device(ea_ctx *c) {
  CU(cudaSetDevice(c->device));
  return EA_OK;
}

}  // namespace

namespace eagb {
// Lets other translation units of the library report through ea_last_error().
void set_last_error(const char *msg) { g_err = msg; }
}  // namespace eagb

static void prof_collect(ea_ctx *c) {
  for (int k = 0; k < EA_K_COUNT; ++k) {
    for (auto &p : c->prof_ev[k]) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, p.first, p.second) == cudaSuccess) {
        c->prof_ms[k] += ms;
        c->prof_n[k] += 1;
      }
      cudaEventDestroy(p.first);
      cudaEventDestroy(p.second);
    }
    c->prof_ev[k].clear();
  }
}


// Driver entry points of the green-context API, looked up at run time so
// that the library needs no link to the driver library.
static void *drv_fn(const char *name) {
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &fn, CUDA_VERSION, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return fn;
}

// Splits the device into nsm SMs for the cluster-uniform generator and the
// rest for the job, and creates the two streams there.
static int make_partition(ea_ctx *c, int nsm) {
  using GetRes = CUresult (*)(CUdevice, CUdevResource *, CUdevResourceType);
  using Split = CUresult (*)(CUdevResource *, unsigned *, const CUdevResource *, CUdevResource *, unsigned, unsigned);
  using GenDesc = CUresult (*)(CUdevResourceDesc *, CUdevResource *, unsigned);
  using GCreate = CUresult (*)(CUgreenCtx *, CUdevResourceDesc, CUdevice, unsigned);
  using GStream = CUresult (*)(CUstream *, CUgreenCtx, unsigned, int);
  using DevGet = CUresult (*)(CUdevice *, int);
  auto devget = (DevGet)drv_fn("cuDeviceGet");
  auto getres = (GetRes)drv_fn("cuDeviceGetDevResource");
  auto split = (Split)drv_fn("cuDevSmResourceSplitByCount");
  auto gendesc = (GenDesc)drv_fn("cuDevResourceGenerateDesc");
  auto gcreate = (GCreate)drv_fn("cuGreenCtxCreate");
  auto gstream = (GStream)drv_fn("cuGreenCtxStreamCreate");
  if (!devget || !getres || !split || !gendesc || !gcreate || !gstream)
    return fail(EA_ERR_CUDA, "green contexts are not available from this driver");
  CUdevice dev;
  CUdevResource all, grp, rest;
  unsigned ng = 1;
  CUdevResourceDesc d[2];
  CUstream s[2];
  if (devget(&dev, c->device) || getres(dev, &all, CU_DEV_RESOURCE_TYPE_SM) ||
      split(&grp, &ng, &all, &rest, 0, (unsigned)nsm) || ng != 1 || gendesc(&d[0], &grp, 1) ||
      gendesc(&d[1], &rest, 1) || gcreate(&c->part[0], d[0], dev, CU_GREEN_CTX_DEFAULT_STREAM) ||
      gcreate(&c->part[1], d[1], dev, CU_GREEN_CTX_DEFAULT_STREAM) ||
      gstream(&s[0], c->part[0], CU_STREAM_NON_BLOCKING, 0) || gstream(&s[1], c->part[1], CU_STREAM_NON_BLOCKING, 0))
    return fail(EA_ERR_CUDA, "SM partition of %d SMs failed", nsm);
  c->rs = (cudaStream_t)s[0];
  c->st = (cudaStream_t)s[1];
  c->part_sms = (int)grp.sm.smCount;
  return EA_OK;
}

static void drop_partition(ea_ctx *c) {
  using GDestroy = CUresult (*)(CUgreenCtx);
  auto gdestroy = (GDestroy)drv_fn("cuGreenCtxDestroy");
  for (CUgreenCtx &g : c->part)
    if (g && gdestroy) { gdestroy(g); g = nullptr; }
}


extern "C" {

const char *ea_last_error(void) { return g_err.c_str(); }
int ea_version(void) { return EA_VERSION; }

int ea_device_count(int32_t *count) {
  if (!count) return fail(EA_ERR_ARG, "null argument");
  int n = 0;
  CU(cudaGetDeviceCount(&n));
  *count = n;
  return EA_OK;
}

// ---------------------------------------------------------------------------
// Host-side set-up
// ---------------------------------------------------------------------------
int ea_host_seeds(uint64_t master_J, uint64_t master_u, uint64_t master_MC, uint64_t master_cluster,
                  const int32_t *list_samples, int32_t nsamples, int32_t nrep, uint64_t *seeds_J,
                  uint64_t *seeds_u, uint64_t *seeds_MC) {
  (void)master_cluster;
  if (nsamples < 1 || nsamples > 32 || nrep < 1 || nrep > 64) return fail(EA_ERR_ARG, "bad sizes");
  if (!master_J || !master_u || !master_MC) return fail(EA_ERR_ARG, "master seeds must be nonzero");
  uint64_t tmp[64];
  std::vector<int32_t> ls(nsamples);
  for (int i = 0; i < nsamples; ++i) {
    ls[i] = list_samples ? list_samples[i] : i;
    if (ls[i] < 0 || ls[i] >= 32 || (i && ls[i] <= ls[i - 1])) return fail(EA_ERR_ARG, "sample list must be increasing in [0,32)");
  }
  // generate_seed_vectors (ini.c:32-59)
  seeds_from_one(master_J, tmp, 32);
  for (int i = 0; i < nsamples; ++i) seeds_J[i] = tmp[ls[i]];
  seeds_from_one(master_u, tmp, 32);
  for (int i = 0; i < nsamples; ++i) seeds_u[i] = tmp[ls[i]];
  seeds_from_one(master_MC, tmp, nrep);
  for (int r = 0; r < nrep; ++r) seeds_MC[r] = tmp[r];
  return EA_OK;
}

int ea_host_generators(const uint64_t *seeds_MC, const int32_t *list_samples, int32_t nsamples, int32_t nrep,
                       uint64_t seed_cluster, ea_generators *gen, ea_hq *pt_out) {
  if (!seeds_MC || !gen || !pt_out || nrep < 1 || nrep > 64 || nsamples < 1 || nsamples > 32)
    return fail(EA_ERR_ARG, "bad arguments");
  if (!seed_cluster) return fail(EA_ERR_ARG, "cluster seed must be nonzero");
  std::memset(gen, 0, sizeof(*gen));
  // Init_Random (ini.c:61-101)
  hq_seed(gen->rc, seed_cluster);
  for (int r = 0; r < nrep; ++r) init_generators(seeds_MC[r], gen->prc[r], gen->xo[r], gen->keys[r]);
  uint64_t tmp[32];
  for (int r = 0; r < nrep; ++r) {
    seeds_from_one(seeds_MC[r], tmp, 32);
    for (int i = 0; i < nsamples; ++i) {
      const int s = list_samples ? list_samples[i] : i;
      // the reference passes this seed through an int (ini.c:63,90)
      const int32_t s32 = (int32_t)(uint32_t)tmp[s];
      hq_seed(pt_out[(size_t)i * nrep + r], (uint64_t)(int64_t)s32);
    }
  }
  gen->cuda_rng_offset = 0;
  gen->seed_cluster = seed_cluster;
  return EA_OK;
}

int ea_host_init_spins(const ea_geom *gp, uint64_t seed_u, uint64_t *even, uint64_t *odd) {
  Geometry g;
  if (!gp || !g.set(*gp) || !even || !odd) return fail(EA_ERR_ARG, "bad geometry");
  std::vector<uint8_t> uu;
  init_spin_bytes(g, seed_u, uu);
  for (int r = 0; r < g.NR; ++r)
    for (int c = 0; c < g.NB; ++c) pack_clone(g, uu.data() + ((size_t)r * g.NB + c) * g.V, r, c, even, odd);
  return EA_OK;
}

int ea_host_init_couplings(const ea_geom *gp, uint64_t seed_J, uint8_t *J6, uint64_t *Jw, int32_t *countJ) {
  Geometry g;
  if (!gp || !g.set(*gp) || !Jw) return fail(EA_ERR_ARG, "bad geometry");
  std::vector<uint8_t> tmp;
  if (!J6) { tmp.resize((size_t)6 * g.V); J6 = tmp.data(); }
  const int cnt = init_couplings(g, seed_J, J6);
  pack_couplings(g, J6, Jw);
  if (countJ) *countJ = cnt;
  return EA_OK;
}

int ea_host_unpack_replica(const ea_geom *gp, const uint64_t *even, const uint64_t *odd, int32_t rep, uint8_t *u) {
  Geometry g;
  if (!gp || !g.set(*gp) || rep < 0 || rep >= g.NR) return fail(EA_ERR_ARG, "bad arguments");
  for (int c = 0; c < g.NB; ++c) unpack_clone(g, even, odd, rep, c, u + (size_t)c * g.V);
  return EA_OK;
}

int ea_host_pack_replica(const ea_geom *gp, const uint8_t *u, int32_t rep, uint64_t *even, uint64_t *odd) {
  Geometry g;
  if (!gp || !g.set(*gp) || rep < 0 || rep >= g.NR) return fail(EA_ERR_ARG, "bad arguments");
  for (int c = 0; c < g.NB; ++c) pack_clone(g, u + (size_t)c * g.V, rep, c, even, odd);
  return EA_OK;
}

int ea_host_scalar_energy(const ea_geom *gp, const uint8_t *u, const uint8_t *J6, int32_t *E) {
  Geometry g;
  if (!gp || !g.set(*gp) || !u || !J6 || !E) return fail(EA_ERR_ARG, "bad arguments");
  *E = scalar_energy(g, u, J6);
  return EA_OK;
}

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
int ea_create(const ea_geom *gp, int32_t device, ea_ctx **out) {
  if (!gp || !out) return fail(EA_ERR_ARG, "null argument");
  ea_ctx *c = new ea_ctx();
  if (!c->g.set(*gp)) { delete c; return fail(EA_ERR_ARG, "geometry: L, Lz multiples of 8, 2<=NB<=255, 1<=nsamples<=32"); }
  const Geometry &g = c->g;
  c->device = device;
  int rc;
  const int kt = choose_kt(g);
  if (!kt || (g.NR != 8 && g.NR != 4 && g.NR != 2)) {
    delete c;
    return fail(EA_ERR_ARG, "unsupported NR=%d / NB=%d (thresholds of every temperature must fit in SMEM)", g.NR, g.NB);
  }
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete c; return fail(EA_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e)); }
  e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return fail(EA_ERR_CUDA, "stream: %s", cudaGetErrorString(e)); }
  JobDev &j = c->j;
  j.NB = g.NB; j.NR = g.NR; j.ns = g.ns; j.half = g.half; j.msc_l = g.msc_l; j.msc_s = g.msc_s;
  j.msc_lz = g.msc_lz; j.L = g.L; j.Lz = g.Lz; j.V = g.V; j.bc = g.bc; j.kt = kt;
  j.ntiles = (g.half + kt - 1) / kt;
  j.cc_xq = (int)(((1ULL << 32) - 1 + (uint64_t)g.L) % (uint64_t)g.L);
  set_dividers(j);
  const size_t nsr = (size_t)g.ns * g.NR;
#define OWN(p, n) if ((rc = own(c, p, n)) != EA_OK) { ea_destroy(c); return rc; }
  OWN(j.spins, g.ns * g.words_per_sample());
  { unsigned long long *p; OWN(p, (size_t)g.ns * 12 * g.half); j.J = p; }
  { int32_t *p; OWN(p, (size_t)12 * g.half); j.nbidx = p; }
  { uint8_t *p; OWN(p, (size_t)2 * g.half); j.nbflag = p; }
  { unsigned long long *p; OWN(p, (size_t)g.NB * 256); j.cum = p; }
  { uint16_t *p; OWN(p, (size_t)g.NB * 256); j.pre = p; }
  OWN(j.wctb, nsr * g.NB);
  OWN(j.wbtc, nsr * g.NB);
  OWN(j.ctr, (size_t)g.NR);
  { uint32_t *p; OWN(p, (size_t)g.NR); j.keys = p; }
  OWN(j.prc, (size_t)g.NR);
  OWN(j.xo, (size_t)g.NR);
  OWN(j.iter, 1);
  OWN(j.epart, (size_t)j.ntiles * nsr * g.NB);
  OWN(j.E, nsr * g.NB);
  OWN(j.pt, nsr);
  { double *p; OWN(p, (size_t)g.NB); j.betas = p; }
  { int32_t *p; OWN(p, (size_t)g.NB); j.expoff = p; }
  OWN(j.acc, nsr * (g.NB - 1));
  OWN(j.att, nsr * (g.NB - 1));
  OWN(j.accraw, nsr * (g.NB - 1));
  OWN(j.inexact, 1);
  OWN(j.rc, 1);
  OWN(j.pairs, 4);
  OWN(c->avgE, nsr * g.NB);
  j.avgE = c->avgE;
#undef OWN
  std::vector<int32_t> idx;
  std::vector<uint8_t> fl;
  neighbour_tables(g, idx, fl);
  CU(cudaMemcpyAsync((void *)j.nbidx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync((void *)j.nbflag, fl.data(), fl.size(), cudaMemcpyHostToDevice, c->st));
  if ((rc = ea_set_permutations(c, nullptr)) != EA_OK) { ea_destroy(c); return rc; }
  CU(cudaStreamSynchronize(c->st));
  if ((rc = ea_set_rng_sms(c, -1)) != EA_OK) { ea_destroy(c); return rc; }
  *out = c;
  return EA_OK;
}

int ea_get_rng_sms(const ea_ctx *c, int32_t *nsm) {
  if (!c || !nsm) return fail(EA_ERR_ARG, "null argument");
  *nsm = c->part_sms;
  return EA_OK;
}

int ea_set_rng_sms(ea_ctx *c, int32_t nsm) {
  if (check(c)) return EA_ERR_ARG;
  if (c->gen) return fail(EA_ERR_STATE, "the SM split is set before the first cluster move");
  if (set_device(c)) return EA_ERR_CUDA;
  const Geometry &g = c->g;
  int nsms = 0;
  CU(cudaDeviceGetAttribute(&nsms, cudaDevAttrMultiProcessorCount, c->device));
  if (nsm < 0) nsm = (2.0 * g.V * g.NB * g.ns >= (double)(1 << 24) && nsms >= 128) ? 32 : 0;
  if (nsm >= nsms) return fail(EA_ERR_ARG, "SM split %d of %d SMs", nsm, nsms);
  if (nsm == c->part_sms) return EA_OK;
  CU(cudaStreamSynchronize(c->st));
  if (c->rs) CU(cudaStreamSynchronize(c->rs));
  cudaStream_t old_st = c->st, old_rs = c->rs;
  CUgreenCtx old_part[2] = {c->part[0], c->part[1]};
  c->part[0] = c->part[1] = nullptr;
  c->rs = nullptr;
  int rc = EA_OK;
  if (nsm > 0) {
    rc = make_partition(c, nsm);
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = fail(EA_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
    c->part_sms = 0;
  }
  if (rc != EA_OK) {
    drop_partition(c);
    c->st = old_st; c->rs = old_rs;
    c->part[0] = old_part[0]; c->part[1] = old_part[1];
    return rc;
  }
  if (old_rs) cudaStreamDestroy(old_rs);
  cudaStreamDestroy(old_st);
  using GDestroy = CUresult (*)(CUgreenCtx);
  auto gdestroy = (GDestroy)drv_fn("cuGreenCtxDestroy");
  for (CUgreenCtx gx : old_part)
    if (gx && gdestroy) gdestroy(gx);
  return EA_OK;
}

int ea_destroy(ea_ctx *c) {
  if (!c) return EA_OK;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->rs) cudaStreamSynchronize(c->rs);
  if (c->gen) curandDestroyGenerator(c->gen);
  prof_collect(c);
  for (void *p : c->owned) cudaFree(p);
  for (auto &set : c->U)
    for (double *u : set)
      if (u) cudaFree(u);
  for (int s = 0; s < 2; ++s) {
    if (c->drawn[s]) cudaEventDestroy(c->drawn[s]);
    if (c->used[s]) cudaEventDestroy(c->used[s]);
  }
  if (c->cs) cudaStreamSynchronize(c->cs);
  if (c->staged) cudaEventDestroy(c->staged);
  if (c->stage_free) cudaEventDestroy(c->stage_free);
  if (c->stage) cudaFree(c->stage);
  if (c->cs) cudaStreamDestroy(c->cs);
  if (c->rs) cudaStreamDestroy(c->rs);
  if (c->st) cudaStreamDestroy(c->st);
  c->st = nullptr;
  drop_partition(c);
  if (c->label) cudaFree(c->label);
  if (c->sel) cudaFree(c->sel);
  if (c->Q) cudaFree(c->Q);
  if (c->hist) cudaFree(c->hist);
  if (c->exptab) cudaFree(c->exptab);
  delete c;
  return EA_OK;
}

int ea_get_geom(const ea_ctx *c, ea_geom *g) {
  if (!c || !g) return fail(EA_ERR_ARG, "null argument");
  g->L = c->g.L; g->Lz = c->g.Lz; g->nbetas = c->g.NB; g->nrep = c->g.NR; g->nsamples = c->g.ns; g->bc = c->g.bc;
  return EA_OK;
}

int ea_sync(ea_ctx *c) {
  if (check(c)) return EA_ERR_ARG;
  CU(cudaStreamSynchronize(c->st));
  if (c->rs) CU(cudaStreamSynchronize(c->rs));
  if (c->cs) CU(cudaStreamSynchronize(c->cs));
  return EA_OK;
}

int ea_join(ea_ctx *c) {
  if (check(c)) return EA_ERR_ARG;
  if (!c->rs) return EA_OK;
  if (set_device(c)) return EA_ERR_CUDA;
  cudaEvent_t e;
  CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CU(cudaEventRecord(e, c->rs));
  CU(cudaStreamWaitEvent(c->st, e, 0));
  CU(cudaEventDestroy(e));
  return EA_OK;
}

int ea_get_stream(ea_ctx *c, void **stream) {
  if (check(c) || !stream) return fail(EA_ERR_ARG, "null argument");
  *stream = (void *)c->st;
  return EA_OK;
}

int ea_set_temperatures(ea_ctx *c, const double *betas, const uint64_t *cum) {
  if (check(c) || !betas || !cum) return fail(EA_ERR_ARG, "null argument");
  const Geometry &g = c->g;
  for (int i = 0; i + 1 < g.NB; ++i)
    if (betas[i] < betas[i + 1]) return fail(EA_ERR_ARG, "betas must be sorted from largest to smallest");
  std::vector<uint16_t> pre((size_t)g.NB * 256);
  for (int b = 0; b < g.NB; ++b) {
    if (cum[(size_t)b * 256 + 255] != ~0ULL) return fail(EA_ERR_ARG, "threshold 255 of beta %d is not 2^64-1", b);
    for (int n = 1; n < 256; ++n)
      if (cum[(size_t)b * 256 + n] < cum[(size_t)b * 256 + n - 1]) return fail(EA_ERR_ARG, "thresholds of beta %d decrease", b);
    presearch8(cum + (size_t)b * 256, pre.data() + (size_t)b * 256);
  }
  std::vector<double> tab;
  pt_exp_table(betas, g.NB, tab, c->expoff);
  if (set_device(c)) return EA_ERR_CUDA;
  CU(cudaMemcpyAsync((void *)c->j.cum, cum, sizeof(uint64_t) * 256 * g.NB, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync((void *)c->j.pre, pre.data(), pre.size() * 2, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync((void *)c->j.betas, betas, sizeof(double) * g.NB, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync((void *)c->j.expoff, c->expoff.data(), sizeof(int32_t) * g.NB, cudaMemcpyHostToDevice, c->st));
  CU(cudaStreamSynchronize(c->st));
  if (c->exptab) cudaFree(c->exptab);
  c->exptab = nullptr;
  CU(dalloc(c->exptab, tab.size()));
  CU(cudaMemcpy(c->exptab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
  c->j.exptab = c->exptab;
  c->have_temps = true;
  return EA_OK;
}

int ea_set_spins(ea_ctx *c, int32_t s, const uint64_t *even, const uint64_t *odd) {
  if (check(c) || s < 0 || s >= c->g.ns || !even || !odd) return fail(EA_ERR_ARG, "bad arguments");
  const size_t n = c->g.words_per_parity();
  if (set_device(c)) return EA_ERR_CUDA;
  unsigned long long *base = c->j.spins + (size_t)s * 2 * n;
  CU(cudaMemcpyAsync(base, even, n * 8, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync(base + n, odd, n * 8, cudaMemcpyHostToDevice, c->st));
  CU(cudaStreamSynchronize(c->st));
  c->energies_fresh = false;
  return EA_OK;
}

int ea_stage_spins_async(ea_ctx *c, const uint64_t *all) {
  if (check(c) || !all) return fail(EA_ERR_ARG, "bad arguments");
  if (set_device(c)) return EA_ERR_CUDA;
  const size_t n = (size_t)c->g.ns * c->g.words_per_sample();
  if (!c->stage) {
    CU(cudaStreamCreateWithFlags(&c->cs, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&c->staged, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&c->stage_free, cudaEventDisableTiming));
    CU(dalloc(c->stage, n));
    CU(cudaEventRecord(c->stage_free, c->st));
  }
  // the buffer is reused once the previous state has been moved out of it
  CU(cudaStreamWaitEvent(c->cs, c->stage_free, 0));
  CU(cudaMemcpyAsync(c->stage, all, n * 8, cudaMemcpyHostToDevice, c->cs));
  CU(cudaEventRecord(c->staged, c->cs));
  c->stage_pending = true;
  return EA_OK;
}

int ea_commit_staged_spins(ea_ctx *c) {
  if (check(c)) return fail(EA_ERR_ARG, "bad arguments");
  if (!c->stage_pending) return fail(EA_ERR_STATE, "no staged spin state");
  if (set_device(c)) return EA_ERR_CUDA;
  const size_t n = (size_t)c->g.ns * c->g.words_per_sample();
  CU(cudaStreamWaitEvent(c->st, c->staged, 0));
  CU(cudaMemcpyAsync(c->j.spins, c->stage, n * 8, cudaMemcpyDeviceToDevice, c->st));
  CU(cudaEventRecord(c->stage_free, c->st));
  c->stage_pending = false;
  c->energies_fresh = false;
  return EA_OK;
}

int ea_upload_spins_async(ea_ctx *c, const uint64_t *all) {
  const int rc = ea_stage_spins_async(c, all);
  return rc ? rc : ea_commit_staged_spins(c);
}

int ea_get_spins(ea_ctx *c, int32_t s, uint64_t *even, uint64_t *odd) {
  if (check(c) || s < 0 || s >= c->g.ns || !even || !odd) return fail(EA_ERR_ARG, "bad arguments");
  const size_t n = c->g.words_per_parity();
  if (set_device(c)) return EA_ERR_CUDA;
  const unsigned long long *base = c->j.spins + (size_t)s * 2 * n;
  CU(cudaMemcpyAsync(even, base, n * 8, cudaMemcpyDeviceToHost, c->st));
  CU(cudaMemcpyAsync(odd, base + n, n * 8, cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

int ea_set_couplings(ea_ctx *c, int32_t s, const uint64_t *Jw) {
  if (check(c) || s < 0 || s >= c->g.ns || !Jw) return fail(EA_ERR_ARG, "bad arguments");
  if (set_device(c)) return EA_ERR_CUDA;
  const size_t n = (size_t)12 * c->g.half;
  CU(cudaMemcpyAsync((void *)(c->j.J + (size_t)s * n), Jw, n * 8, cudaMemcpyHostToDevice, c->st));
  CU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

int ea_set_generators(ea_ctx *c, const ea_generators *gen, const ea_hq *pt) {
  if (check(c) || !gen || !pt) return fail(EA_ERR_ARG, "null argument");
  const Geometry &g = c->g;
  if (set_device(c)) return EA_ERR_CUDA;
  CU(cudaMemcpyAsync(c->j.prc, gen->prc, sizeof(ea_hq) * g.NR, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync(c->j.xo, gen->xo, sizeof(ea_xoshiro) * g.NR, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync((void *)c->j.keys, gen->keys, sizeof(uint32_t) * g.NR, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync(c->j.rc, &gen->rc, sizeof(ea_hq), cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync(c->j.pt, pt, sizeof(ea_hq) * g.ns * g.NR, cudaMemcpyHostToDevice, c->st));
  CU(cudaStreamSynchronize(c->st));
  // The same cluster seed and offset as the job's own continue its generator
  // (uniforms drawn ahead included), as the reference process keeps its
  // generator across bins; other values start a new generator there, as
  // ClusterInit does on a restart.
  if (c->gen && (gen->seed_cluster != c->seed_cluster || gen->cuda_rng_offset != c->cuda_rng_offset)) {
    CU(cudaStreamSynchronize(c->rs));
    curandDestroyGenerator(c->gen);
    c->gen = nullptr;
    c->ready = 0;
  }
  c->cuda_rng_offset = gen->cuda_rng_offset;
  c->seed_cluster = gen->seed_cluster;
  return EA_OK;
}

int ea_get_generators(ea_ctx *c, ea_generators *gen, ea_hq *pt) {
  if (check(c) || !gen) return fail(EA_ERR_ARG, "null argument");
  const Geometry &g = c->g;
  if (set_device(c)) return EA_ERR_CUDA;
  std::memset(gen, 0, sizeof(*gen));
  CU(cudaMemcpyAsync(gen->prc, c->j.prc, sizeof(ea_hq) * g.NR, cudaMemcpyDeviceToHost, c->st));
  CU(cudaMemcpyAsync(gen->xo, c->j.xo, sizeof(ea_xoshiro) * g.NR, cudaMemcpyDeviceToHost, c->st));
  CU(cudaMemcpyAsync(gen->keys, c->j.keys, sizeof(uint32_t) * g.NR, cudaMemcpyDeviceToHost, c->st));
  CU(cudaMemcpyAsync(&gen->rc, c->j.rc, sizeof(ea_hq), cudaMemcpyDeviceToHost, c->st));
  if (pt) CU(cudaMemcpyAsync(pt, c->j.pt, sizeof(ea_hq) * g.ns * g.NR, cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  gen->cuda_rng_offset = c->cuda_rng_offset;
  gen->seed_cluster = c->seed_cluster;
  return EA_OK;
}

int ea_set_permutations(ea_ctx *c, const uint8_t *wctb) {
  if (check(c)) return EA_ERR_ARG;
  const Geometry &g = c->g;
  const size_t n = (size_t)g.ns * g.NR * g.NB;
  std::vector<uint8_t> a(n), b(n);
  for (size_t o = 0; o < (size_t)g.ns * g.NR; ++o) {
    std::vector<int> seen(g.NB, 0);
    for (int i = 0; i < g.NB; ++i) {
      const uint8_t v = wctb ? wctb[o * g.NB + i] : (uint8_t)i;
      if (v >= g.NB || seen[v]++) return fail(EA_ERR_ARG, "which_clon_this_beta is not a permutation");
      a[o * g.NB + i] = v;
      b[o * g.NB + v] = (uint8_t)i;
    }
  }
  if (set_device(c)) return EA_ERR_CUDA;
  CU(cudaMemcpyAsync(c->j.wctb, a.data(), n, cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync(c->j.wbtc, b.data(), n, cudaMemcpyHostToDevice, c->st));
  CU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

int ea_get_permutations(ea_ctx *c, uint8_t *wctb, uint8_t *wbtc) {
  if (check(c)) return EA_ERR_ARG;
  const size_t n = (size_t)c->g.ns * c->g.NR * c->g.NB;
  if (set_device(c)) return EA_ERR_CUDA;
  if (wctb) CU(cudaMemcpyAsync(wctb, c->j.wctb, n, cudaMemcpyDeviceToHost, c->st));
  if (wbtc) CU(cudaMemcpyAsync(wbtc, c->j.wbtc, n, cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

int ea_get_pt_stats(ea_ctx *c, double *acc, double *att, double *accraw) {
  if (check(c)) return EA_ERR_ARG;
  const size_t n = (size_t)c->g.ns * c->g.NR * (c->g.NB - 1);
  if (set_device(c)) return EA_ERR_CUDA;
  if (acc) CU(cudaMemcpyAsync(acc, c->j.acc, n * 8, cudaMemcpyDeviceToHost, c->st));
  if (att) CU(cudaMemcpyAsync(att, c->j.att, n * 8, cudaMemcpyDeviceToHost, c->st));
  if (accraw) CU(cudaMemcpyAsync(accraw, c->j.accraw, n * 8, cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

int ea_reset_pt_stats(ea_ctx *c) {
  if (check(c)) return EA_ERR_ARG;
  const size_t n = (size_t)c->g.ns * c->g.NR * (c->g.NB - 1);
  if (set_device(c)) return EA_ERR_CUDA;
  CU(cudaMemsetAsync(c->j.acc, 0, n * 8, c->st));
  CU(cudaMemsetAsync(c->j.att, 0, n * 8, c->st));
  CU(cudaMemsetAsync(c->j.accraw, 0, n * 8, c->st));
  return EA_OK;
}

int ea_set_counter(ea_ctx *c, int64_t iter, uint32_t jobid) {
  if (check(c) || iter < 0 || jobid >= (1u << 14)) return fail(EA_ERR_ARG, "iter >= 0 and job id < 2^14");
  if (set_device(c)) return EA_ERR_CUDA;
  long long v = iter;
  CU(cudaMemcpyAsync(c->j.iter, &v, 8, cudaMemcpyHostToDevice, c->st));
  CU(cudaStreamSynchronize(c->st));
  c->j.jobid = jobid;
  return EA_OK;
}

int ea_get_counter(ea_ctx *c, int64_t *iter) {
  if (check(c) || !iter) return EA_ERR_ARG;
  if (set_device(c)) return EA_ERR_CUDA;
  long long v = 0;
  CU(cudaMemcpyAsync(&v, c->j.iter, 8, cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  *iter = v;
  return EA_OK;
}

// ---------------------------------------------------------------------------
// Hot path
// ---------------------------------------------------------------------------
// Event pair around one launch when profiling is on (ea_profile).
static cudaEvent_t prof_begin(ea_ctx *c, cudaStream_t st = nullptr) {
  if (!c->prof_on) return nullptr;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  cudaEventRecord(e, st ? st : c->st);
  return e;
}

static void prof_end(ea_ctx *c, int kind, cudaEvent_t b, cudaStream_t st = nullptr) {
  if (!b) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, st ? st : c->st);
  c->prof_ev[kind].push_back({b, e});
}

static int mc(ea_ctx *c, int n) {
  for (int sw = 0; sw < n; ++sw)
    for (int p = 0; p < 2; ++p) {
      CU(launch_fill_bits(c->j, p, c->st));
      cudaEvent_t b = prof_begin(c);
      CU(launch_sweep(c->j, p, sw == n - 1 && p == 1, c->st));
      prof_end(c, EA_K_SWEEP, b);
    }
  if (n > 0) {
    CU(launch_energy_reduce(c->j, c->st));
    c->energies_fresh = true;
  }
  return EA_OK;
}

int ea_monte_carlo(ea_ctx *c, int32_t nsweeps) {
  if (check(c) || nsweeps < 0) return fail(EA_ERR_ARG, "bad arguments");
  if (!c->have_temps) return fail(EA_ERR_STATE, "temperatures not set");
  if (set_device(c)) return EA_ERR_CUDA;
  return mc(c, nsweeps);
}

static int measure(ea_ctx *c) {
  cudaEvent_t b = prof_begin(c);
  CU(launch_energy(c->j, c->st));
  CU(launch_energy_reduce(c->j, c->st));
  prof_end(c, EA_K_ENERGY, b);
  c->energies_fresh = true;
  return EA_OK;
}

int ea_measure_energy(ea_ctx *c, int32_t *out) {
  if (check(c)) return EA_ERR_ARG;
  if (set_device(c)) return EA_ERR_CUDA;
  int rc = measure(c);
  if (rc) return rc;
  if (out) {
    CU(cudaMemcpyAsync(out, c->j.E, sizeof(int32_t) * c->g.ns * c->g.NR * c->g.NB, cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
  }
  return EA_OK;
}

static int pt(ea_ctx *c) {
  cudaEvent_t b = prof_begin(c);
  CU(launch_pt(c->j, c->st));
  prof_end(c, EA_K_PT, b);
  return EA_OK;
}

int ea_parallel_tempering(ea_ctx *c) {
  if (check(c)) return EA_ERR_ARG;
  if (!c->have_temps) return fail(EA_ERR_STATE, "temperatures not set");
  if (!c->energies_fresh) return fail(EA_ERR_STATE, "no energies of the current state (run ea_monte_carlo or ea_measure_energy)");
  if (set_device(c)) return EA_ERR_CUDA;
  return pt(c);
}

static int ensure_cluster(ea_ctx *c, int nclust) {
  const Geometry &g = c->g;
  if (!c->rs) {
    int least = 0, greatest = 0;
    CU(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CU(cudaStreamCreateWithPriority(&c->rs, cudaStreamNonBlocking, greatest));
  }
  if (!c->drawn[0]) {
    for (int s = 0; s < 2; ++s) {
      CU(cudaEventCreateWithFlags(&c->drawn[s], cudaEventDisableTiming));
      CU(cudaEventCreateWithFlags(&c->used[s], cudaEventDisableTiming));
    }
  }
  for (auto &set : c->U)
    for (double *&u : set)
      if (!u) CU(dalloc(u, (size_t)g.V * g.NB * g.ns));
  if (nclust > c->nclust_cap) {
    CU(cudaStreamSynchronize(c->st));
    if (c->label) cudaFree(c->label);
    if (c->sel) cudaFree(c->sel);
    if (c->Q) cudaFree(c->Q);
    c->label = nullptr; c->sel = nullptr; c->Q = nullptr;
    CU(dalloc(c->label, (size_t)g.V * nclust * g.ns));
    CU(dalloc(c->sel, (size_t)g.V / 32 * nclust * g.ns));
    CU(dalloc(c->Q, (size_t)2 * g.half * nclust * g.ns));
    c->nclust_cap = nclust;
  }
  c->j.label = c->label;
  c->j.sel = c->sel;
  c->j.Q = c->Q;
  c->j.nclust = nclust;
  set_dividers(c->j);
  if (!c->gen) {
    // ClusterInit (HoudayerXEA.cu:174-178): default pseudo generator (XORWOW),
    // seed_Cluster, and the offset already consumed.
    CR(curandCreateGenerator(&c->gen, CURAND_RNG_PSEUDO_DEFAULT));
    CR(curandSetPseudoRandomGeneratorSeed(c->gen, (unsigned long long)c->seed_cluster));
    if (c->cuda_rng_offset > 0) CR(curandSetGeneratorOffset(c->gen, c->cuda_rng_offset));
    CR(curandSetStream(c->gen, c->rs));
    c->ready = 0;
  }
  return EA_OK;
}

static int norm_nclust(const Geometry &g, int nclust) {
  if (nclust <= 0) nclust = (int)std::lround(g.NB * 0.5);
  return nclust > g.NB ? g.NB : nclust;
}

// ClusterStep's uniforms (HoudayerXEA.cu:189-195) for both groups of one move,
// V*NB*nsamples doubles per group in the reference's call sizes, into set
// `set` once the move that last read it has finished.
static int houdayer_draw(ea_ctx *c, int set) {
  const Geometry &g = c->g;
  const size_t tot = (size_t)g.V * g.NB * g.ns;
  CU(cudaStreamWaitEvent(c->rs, c->used[set], 0));
  cudaEvent_t b = prof_begin(c, c->rs);
  for (int grp = 0; grp < 2; ++grp) CR(curandGenerateUniformDouble(c->gen, c->U[set][grp], tot));
  prof_end(c, EA_K_RNG, b, c->rs);
  CU(cudaEventRecord(c->drawn[set], c->rs));
  return EA_OK;
}

// Everything of a move that happens before its kernels: buffers, the
// generator, and the uniforms of this move (and of the next one, drawn ahead).
static int houdayer_prepare(ea_ctx *c, int nclust) {
  const Geometry &g = c->g;
  if (g.NR < 4) return fail(EA_ERR_ARG, "the Houdayer move needs at least 2 replicas per group");
  int rc = ensure_cluster(c, norm_nclust(g, nclust));
  if (rc) return rc;
  if (c->ready == 0) {
    if ((rc = houdayer_draw(c, c->cur))) return rc;
    c->ready = 1;
  }
  if (c->ready == 1) {
    if ((rc = houdayer_draw(c, c->cur ^ 1))) return rc;
    c->ready = 2;
  }
  return EA_OK;
}

// After the move's kernels were enqueued on stream s.
static int houdayer_finish(ea_ctx *c, cudaStream_t s) {
  const Geometry &g = c->g;
  CU(cudaEventRecord(c->used[c->cur], s));
  c->cur ^= 1;
  c->ready = 1;
  c->cuda_rng_offset += 2 * (uint64_t)g.V * g.NB * g.ns;
  c->energies_fresh = false;
  return EA_OK;
}

static int houdayer(ea_ctx *c, int nclust) {
  int rc = houdayer_prepare(c, nclust);
  if (rc) return rc;
  CU(launch_houdayer_pairs(c->j, c->st));
  CU(cudaStreamWaitEvent(c->st, c->drawn[c->cur], 0));
  for (int grp = 0; grp < 2; ++grp) {
    JobDev jg = c->j;
    jg.U = c->U[c->cur][grp];
    cudaEvent_t b = prof_begin(c);
    CU(launch_houdayer_group(jg, grp, c->st));
    prof_end(c, EA_K_CLUSTER, b);
  }
  return houdayer_finish(c, c->st);
}

int ea_houdayer(ea_ctx *c, int32_t nclust) {
  if (check(c)) return EA_ERR_ARG;
  if (set_device(c)) return EA_ERR_CUDA;
  return houdayer(c, nclust);
}

int ea_set_cluster_rule(ea_ctx *c, int32_t rule) {
  if (check(c) || (rule != EA_CLUSTER_REFERENCE && rule != EA_CLUSTER_EXACT)) return fail(EA_ERR_ARG, "bad cluster rule");
  const int L = c->g.L;
  c->j.cc_xq = rule == EA_CLUSTER_EXACT ? L - 1 : (int)(((1ULL << 32) - 1 + (uint64_t)L) % (uint64_t)L);
  return EA_OK;
}

static void trw(int itmax, int *frec, int *maxit) {
  for (int f = 1; f <= itmax; ++f)
    if (itmax % f == 0 && itmax / f <= 512) { *frec = f; *maxit = itmax / f; return; }
  *frec = 1; *maxit = itmax;
}

int ea_run_bin(ea_ctx *c, const ea_cadence *cad, double *avgE, uint8_t *hist, int32_t *maxit_trw) {
  if (check(c) || !cad || cad->itmax < 1 || cad->houfr < 1 || cad->mesfr < 1 || cad->ptfr < 0)
    return fail(EA_ERR_ARG, "bad cadence");
  if (!c->have_temps) return fail(EA_ERR_STATE, "temperatures not set");
  if (set_device(c)) return EA_ERR_CUDA;
  const Geometry &g = c->g;
  int frec, maxit;
  trw(cad->itmax, &frec, &maxit);
  const size_t nsr = (size_t)g.ns * g.NR;
  if (maxit > c->hist_cap) {
    if (c->hist) cudaFree(c->hist);
    c->hist = nullptr;
    CU(dalloc(c->hist, nsr * maxit * g.NB));
    c->hist_cap = maxit;
  }
  c->j.hist = c->hist;
  c->j.maxit_trw = maxit;
  CU(cudaMemsetAsync(c->avgE, 0, nsr * g.NB * 8, c->st));
  CU(cudaMemsetAsync(c->hist, 0, nsr * maxit * g.NB, c->st));
  int rc;
  for (int it = 0; it < cad->itmax; ++it) {
    for (int im = 0; im < cad->mesfr; ++im) {
      for (int ih = 0; ih < cad->houfr; ++ih) {
        if ((rc = mc(c, cad->ptfr))) return rc;
        if (!c->energies_fresh && (rc = measure(c))) return rc;
        if ((rc = pt(c))) return rc;
      }
      if (cad->cluster && (rc = houdayer(c, cad->nclust))) return rc;
    }
    if ((rc = measure(c))) return rc;
    CU(launch_measure(c->j, (it % frec == frec - 1) ? it / frec : -1, c->st));
  }
  if (maxit_trw) *maxit_trw = maxit;
  if (!avgE && !hist) return EA_OK;  // nothing to hand back: stay asynchronous
  if (avgE) CU(cudaMemcpyAsync(avgE, c->avgE, nsr * g.NB * 8, cudaMemcpyDeviceToHost, c->st));
  if (hist) CU(cudaMemcpyAsync(hist, c->hist, nsr * maxit * g.NB, cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  return ea_check_exact(c);
}

int ea_check_exact(ea_ctx *c) {
  if (check(c)) return EA_ERR_ARG;
  if (set_device(c)) return EA_ERR_CUDA;
  unsigned long long inex = 0;
  CU(cudaMemcpyAsync(&inex, c->j.inexact, 8, cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  if (inex) return fail(EA_ERR_INEXACT, "%llu tempering decisions fell outside the exact exp table", inex);
  return EA_OK;
}

int ea_profile(ea_ctx *c, int32_t on) {
  if (check(c)) return EA_ERR_ARG;
  if (set_device(c)) return EA_ERR_CUDA;
  CU(cudaStreamSynchronize(c->st));
  prof_collect(c);
  for (int k = 0; k < EA_K_COUNT; ++k) { c->prof_n[k] = 0; c->prof_ms[k] = 0; }
  c->prof_on = on != 0;
  return EA_OK;
}

int ea_kernel_time(ea_ctx *c, int32_t kind, int64_t *launches, double *total_ms) {
  if (check(c) || kind < 0 || kind >= EA_K_COUNT) return fail(EA_ERR_ARG, "bad kernel kind");
  if (set_device(c)) return EA_ERR_CUDA;
  CU(cudaStreamSynchronize(c->st));
  prof_collect(c);
  if (launches) *launches = c->prof_n[kind];
  if (total_ms) *total_ms = c->prof_ms[kind];
  return EA_OK;
}

int ea_curand_uniforms(int32_t device, uint64_t seed, uint64_t offset, uint64_t n, double *out) {
  if (!out) return fail(EA_ERR_ARG, "null output");
  CU(cudaSetDevice(device));
  double *d = nullptr;
  CU(dalloc(d, n));
  curandGenerator_t gen;
  curandStatus_t s = curandCreateGenerator(&gen, CURAND_RNG_PSEUDO_DEFAULT);
  if (s == CURAND_STATUS_SUCCESS) s = curandSetPseudoRandomGeneratorSeed(gen, seed);
  if (s == CURAND_STATUS_SUCCESS && offset) s = curandSetGeneratorOffset(gen, offset);
  if (s == CURAND_STATUS_SUCCESS) s = curandGenerateUniformDouble(gen, d, n);
  curandDestroyGenerator(gen);
  if (s != CURAND_STATUS_SUCCESS) { cudaFree(d); return fail(EA_ERR_CURAND, "curand status %d", (int)s); }
  cudaError_t e = cudaMemcpy(out, d, n * 8, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(EA_ERR_CUDA, "%s", cudaGetErrorString(e));
  return EA_OK;
}


// ---------------------------------------------------------------------------
// Batches: many jobs (geometries, boundary conditions, temperature counts)
// advanced by persistent batched kernels, one launch per step for all of
// them, with the sweep / energy / tempering cycle replayed as a CUDA graph.
// ---------------------------------------------------------------------------
}  // extern "C"

struct ea_batch {
  std::vector<ea_ctx *> jobs;
  int device = 0, NR = 0, KT = 0, NBmax = 0;
  cudaStream_t bs = nullptr;
  cudaEvent_t done = nullptr;
  JobDev *d_jobs = nullptr;
  uint32_t *d_pre = nullptr;
  uint32_t *d_ctr = nullptr;
  std::vector<JobDev> up_jobs;  // JobDev array as last uploaded
  std::vector<uint32_t> up_pre;
  // Uploads are stream-ordered copies from two pinned staging slots, so the
  // work list can change between bins without waiting for the GPU; a slot is
  // reused once the copy that read it has run (up_ev).
  JobDev *h_jobs[2] = {};
  uint32_t *h_pre[2] = {};
  cudaEvent_t up_ev[2] = {};
  int up_slot = 0;
  BatchDev bd{};
  cudaGraphExec_t cycle = nullptr;
  int cycle_ptfr = -1;
  UTable u{};  // uniforms of the current group, by job
  float tuned_ms = 0.f;  // autotuner: two sweeps of the chosen tile width
};

extern "C" {

// Tile width of a job's fused sweep; the energy partial sums follow it.
static int set_tile(ea_ctx *c, int kt) {
  JobDev &j = c->j;
  if (kt == j.kt) return EA_OK;
  const Geometry &g = c->g;
  const size_t smem = sweep_smem_for(g.NB, g.NR, kt);
  if (smem > 227 * 1024) return fail(EA_ERR_ARG, "tile width %d needs %zu bytes of shared memory", kt, smem);
  const int nt = (g.half + kt - 1) / kt;
  if (nt > j.ntiles) {
    int32_t *p = nullptr;
    int rc = own(c, p, (size_t)nt * g.ns * g.NR * g.NB);
    if (rc) return rc;
    j.epart = p;
  }
  j.kt = kt;
  j.ntiles = nt;
  return EA_OK;
}

static int batch_kt(const ea_batch *b, int forced) {
  const int c8[3] = {4, 2, 1}, c4[3] = {8, 4, 2}, c2[3] = {16, 8, 4};
  const int *c = b->NR == 8 ? c8 : b->NR == 4 ? c4 : c2;
  auto fits = [&](int kt) { return batch_sweep_smem(b->NR, kt, b->NBmax) <= 227 * 1024 - 256; };
  if (forced) {
    for (int i = 0; i < 3; ++i)
      if (c[i] == forced && fits(forced)) return forced;
    return 0;
  }
  for (int i = 0; i < 3; ++i) {
    if (!fits(c[i])) continue;
    long tiles = 0;
    for (ea_ctx *x : b->jobs) tiles += (x->g.half + c[i] - 1) / c[i];
    if (tiles >= 4 * 152) return c[i];
  }
  for (int i = 2; i >= 0; --i)
    if (fits(c[i])) return c[i];
  return 0;
}

// Uploads the jobs' descriptors and work lists when they changed.
static int batch_upload(ea_batch *b) {
  const int n = (int)b->jobs.size();
  std::vector<JobDev> hj(n);
  std::vector<uint32_t> hp((size_t)KB_COUNT * (n + 1), 0);
  int slab_threads = 32, flip_smem = 0;
  for (int i = 0; i < n; ++i) {
    hj[i] = b->jobs[i]->j;
    hj[i].U = nullptr;
    uint32_t cnt[KB_COUNT];
    batch_blocks(hj[i], cnt);
    for (int k = 0; k < KB_COUNT; ++k) hp[(size_t)k * (n + 1) + i + 1] = hp[(size_t)k * (n + 1) + i] + cnt[k];
    if (cnt[KB_SLAB]) {
      int D, P, ns;
      slab_shape(hj[i], &D, &P, &ns);
      const int t = hj[i].L * hj[i].L * P;
      if (t > slab_threads) slab_threads = t;
      if ((int)flip_smem_bytes(hj[i]) > flip_smem) flip_smem = (int)flip_smem_bytes(hj[i]);
    }
  }
  const bool same = b->up_jobs.size() == hj.size() &&
                    !std::memcmp(b->up_jobs.data(), hj.data(), sizeof(JobDev) * n) && b->up_pre == hp;
  if (!same) {
    // kernels of earlier bins may still read the arrays: the copies are
    // ordered after them on the batch stream
    const int slot = b->up_slot;
    b->up_slot ^= 1;
    CU(cudaEventSynchronize(b->up_ev[slot]));
    std::memcpy(b->h_jobs[slot], hj.data(), sizeof(JobDev) * n);
    std::memcpy(b->h_pre[slot], hp.data(), sizeof(uint32_t) * hp.size());
    CU(cudaMemcpyAsync(b->d_jobs, b->h_jobs[slot], sizeof(JobDev) * n, cudaMemcpyHostToDevice, b->bs));
    CU(cudaMemcpyAsync(b->d_pre, b->h_pre[slot], sizeof(uint32_t) * hp.size(), cudaMemcpyHostToDevice, b->bs));
    CU(cudaEventRecord(b->up_ev[slot], b->bs));
    b->up_jobs = hj;
    b->up_pre = hp;
  }
  const BatchDev old_bd = b->bd;
  b->bd.jobs = b->d_jobs;
  b->bd.njobs = n;
  for (int k = 0; k < KB_COUNT; ++k) {
    b->bd.pre[k] = b->d_pre + (size_t)k * (n + 1);
    b->bd.total[k] = hp[(size_t)k * (n + 1) + n];
  }
  b->bd.slab_threads = slab_threads;
  b->bd.flip_smem = flip_smem;
  b->bd.ctr = b->d_ctr;
  // chunks of work items a block takes at a time: one heavy item, or several
  // light ones so that the job lookup and the fetch are amortised
  const uint32_t chunk[KB_COUNT] = {1, 4, 1, 4, 4, 1, 4, 4, 1};
  for (int k = 0; k < KB_COUNT; ++k) b->bd.chunk[k] = chunk[k];
  if (b->bd.total[KB_SWEEP] >= 8u * 304u) b->bd.chunk[KB_SWEEP] = 2;
  // the cycle graph holds the descriptor by value
  if (std::memcmp(&old_bd, &b->bd, sizeof(BatchDev)) && b->cycle) {
    cudaGraphExecDestroy(b->cycle);
    b->cycle = nullptr;
  }
  return EA_OK;
}

// Autotuner: times the batched half-sweeps of every tile width that fits, on
// the batch's own jobs, and keeps the fastest.  What the timing sweeps change
// (spin words, half-sweep counter, Philox counters, the two generators that
// feed them) is copied aside on the device first and put back after, so the
// jobs are left exactly as they were.
static int batch_autotune(ea_batch *b, float *best_ms) {
  const int c8[3] = {4, 2, 1}, c4[3] = {8, 4, 2}, c2[3] = {16, 8, 4};
  const int *c = b->NR == 8 ? c8 : b->NR == 4 ? c4 : c2;
  std::vector<int> cand;
  for (int i = 0; i < 3; ++i)
    if (batch_sweep_smem(b->NR, c[i], b->NBmax) <= 227 * 1024 - 256) cand.push_back(c[i]);
  if (cand.empty()) return fail(EA_ERR_ARG, "no tile width fits NB=%d in shared memory", b->NBmax);
  b->KT = cand[0];
  if (cand.size() == 1) return EA_OK;
  struct Part { void *p; size_t n; };
  std::vector<Part> parts;
  size_t total = 0;
  for (ea_ctx *x : b->jobs) {
    const Geometry &g = x->g;
    parts.push_back({x->j.spins, (size_t)g.ns * g.words_per_sample() * 8});
    parts.push_back({x->j.iter, 8});
    parts.push_back({x->j.ctr, sizeof(uint4) * g.NR});
    parts.push_back({x->j.prc, sizeof(ea_hq) * g.NR});
    parts.push_back({x->j.xo, sizeof(ea_xoshiro) * g.NR});
  }
  for (const Part &q : parts) total += (q.n + 255) & ~(size_t)255;
  char *save = nullptr;
  CU(cudaMalloc((void **)&save, total));
  size_t off = 0;
  for (const Part &q : parts) {
    CU(cudaMemcpyAsync(save + off, q.p, q.n, cudaMemcpyDeviceToDevice, b->bs));
    off += (q.n + 255) & ~(size_t)255;
  }
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  int best = cand[0];
  float bms = 1e30f;
  int rc = EA_OK;
  for (int kt : cand) {
    for (ea_ctx *x : b->jobs)
      if ((rc = set_tile(x, kt))) break;
    if (rc || (rc = batch_upload(b))) break;
    if (batch_setup(b->NR, kt) != cudaSuccess) continue;
    float ms = 0.f;
    for (int rep = 0; rep < 2; ++rep) {  // the first pass warms up
      cudaEventRecord(e0, b->bs);
      for (int cyc = 0; cyc < 2; ++cyc)
        for (int p = 0; p < 2; ++p) {
          batch_fill_bits(b->bd, p, b->bs);
          batch_sweep(b->bd, b->NR, kt, b->NBmax, p, p == 1, true, b->bs);
        }
      cudaEventRecord(e1, b->bs);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms, e0, e1);
    }
    if (cudaGetLastError() != cudaSuccess) continue;
    if (ms < bms) { bms = ms; best = kt; }
  }
  off = 0;
  for (const Part &q : parts) {
    cudaMemcpyAsync(q.p, save + off, q.n, cudaMemcpyDeviceToDevice, b->bs);
    off += (q.n + 255) & ~(size_t)255;
  }
  cudaStreamSynchronize(b->bs);
  cudaFree(save);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  b->KT = best;
  for (ea_ctx *x : b->jobs)
    if ((rc = set_tile(x, best))) return rc;
  if (best_ms) *best_ms = bms;
  CU(batch_setup(b->NR, best));
  return batch_upload(b);
}

int ea_batch_create(ea_ctx *const *jobs, int32_t njobs, int32_t tile, ea_batch **out) {
  if (!jobs || !out || njobs < 1 || njobs > kBatchMaxJobs) return fail(EA_ERR_ARG, "1..%d jobs", kBatchMaxJobs);
  ea_batch *b = new ea_batch();
  for (int i = 0; i < njobs; ++i) {
    ea_ctx *c = jobs[i];
    if (!c) { delete b; return fail(EA_ERR_ARG, "null job %d", i); }
    for (ea_ctx *o : b->jobs)
      if (o == c) { delete b; return fail(EA_ERR_ARG, "job %d appears twice", i); }
    if (i && (c->device != b->device || c->g.NR != b->NR)) {
      delete b;
      return fail(EA_ERR_ARG, "the jobs of a batch share the device and the number of replicas");
    }
    b->device = c->device;
    b->NR = c->g.NR;
    if (c->g.NB > b->NBmax) b->NBmax = c->g.NB;
    b->jobs.push_back(c);
  }
  CU(cudaSetDevice(b->device));
  // heaviest work items first (a sweep tile costs ~ NB x samples), so that
  // blocks drawing items in order end together
  std::stable_sort(b->jobs.begin(), b->jobs.end(),
                   [](const ea_ctx *x, const ea_ctx *y) { return x->g.NB * x->g.ns > y->g.NB * y->g.ns; });
  if (tile) {
    b->KT = batch_kt(b, tile);
    if (!b->KT) { delete b; return fail(EA_ERR_ARG, "tile width %d does not fit NR=%d, NB=%d", tile, b->NR, b->NBmax); }
  }
  for (ea_ctx *c : b->jobs) {
    CU(cudaStreamSynchronize(c->st));
    if (tile) {
      int rc = set_tile(c, b->KT);
      if (rc) { delete b; return rc; }
    }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&b->bs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  // room for the largest batch, so that ea_batch_set_jobs never reallocates
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_jobs, sizeof(JobDev) * kBatchMaxJobs);
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_pre, sizeof(uint32_t) * KB_COUNT * (kBatchMaxJobs + 1));
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    e = cudaMallocHost((void **)&b->h_jobs[k], sizeof(JobDev) * kBatchMaxJobs);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&b->h_pre[k], sizeof(uint32_t) * KB_COUNT * (kBatchMaxJobs + 1));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->up_ev[k], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_ctr, sizeof(uint32_t) * KB_COUNT);
  if (e == cudaSuccess) e = cudaMemset(b->d_ctr, 0, sizeof(uint32_t) * KB_COUNT);
  if (e == cudaSuccess && tile) e = batch_setup(b->NR, b->KT);
  if (e != cudaSuccess) { ea_batch_destroy(b); return fail(EA_ERR_CUDA, "batch set-up: %s", cudaGetErrorString(e)); }
  if (!tile) {
    int rc = batch_autotune(b, &b->tuned_ms);
    if (rc) { ea_batch_destroy(b); return rc; }
  }
  *out = b;
  return EA_OK;
}

int ea_batch_destroy(ea_batch *b) {
  if (!b) return EA_OK;
  cudaSetDevice(b->device);
  if (b->bs) cudaStreamSynchronize(b->bs);
  if (b->cycle) cudaGraphExecDestroy(b->cycle);
  if (b->d_jobs) cudaFree(b->d_jobs);
  if (b->d_pre) cudaFree(b->d_pre);
  if (b->d_ctr) cudaFree(b->d_ctr);
  for (int k = 0; k < 2; ++k) {
    if (b->h_jobs[k]) cudaFreeHost(b->h_jobs[k]);
    if (b->h_pre[k]) cudaFreeHost(b->h_pre[k]);
    if (b->up_ev[k]) cudaEventDestroy(b->up_ev[k]);
  }
  if (b->done) cudaEventDestroy(b->done);
  if (b->bs) cudaStreamDestroy(b->bs);
  delete b;
  return EA_OK;
}

int ea_batch_tile(const ea_batch *b, int32_t *tile) {
  if (!b || !tile) return fail(EA_ERR_ARG, "null argument");
  *tile = b->KT;
  return EA_OK;
}

int ea_batch_set_jobs(ea_batch *b, ea_ctx *const *jobs, int32_t njobs) {
  if (!b || !jobs || njobs < 1 || njobs > kBatchMaxJobs) return fail(EA_ERR_ARG, "1..%d jobs", kBatchMaxJobs);
  std::vector<ea_ctx *> nj;
  int nbmax = 0;
  for (int i = 0; i < njobs; ++i) {
    ea_ctx *c = jobs[i];
    if (!c) return fail(EA_ERR_ARG, "null job %d", i);
    if (std::find(nj.begin(), nj.end(), c) != nj.end()) return fail(EA_ERR_ARG, "job %d appears twice", i);
    if (c->device != b->device || c->g.NR != b->NR)
      return fail(EA_ERR_ARG, "the jobs of a batch share the device and the number of replicas");
    if (c->g.NB > nbmax) nbmax = c->g.NB;
    nj.push_back(c);
  }
  if (batch_sweep_smem(b->NR, b->KT, nbmax) > 227 * 1024 - 256)
    return fail(EA_ERR_ARG, "NB=%d does not fit the batch's tile width %d", nbmax, b->KT);
  CU(cudaSetDevice(b->device));
  for (ea_ctx *c : nj) {
    if (std::find(b->jobs.begin(), b->jobs.end(), c) != b->jobs.end()) continue;
    const int rc = set_tile(c, b->KT);
    if (rc) return rc;
  }
  std::stable_sort(nj.begin(), nj.end(),
                   [](const ea_ctx *x, const ea_ctx *y) { return x->g.NB * x->g.ns > y->g.NB * y->g.ns; });
  b->jobs = nj;
  b->NBmax = nbmax;
  return batch_upload(b);
}

// One tempering cycle for every job: ptfr sweeps (energy fused into the last
// odd half-sweep), or an energy pass when ptfr is 0, then the swaps.
static int batch_cycle_launch(ea_batch *b, int ptfr) {
  for (int sw = 0; sw < ptfr; ++sw)
    for (int p = 0; p < 2; ++p) {
      CU(batch_fill_bits(b->bd, p, b->bs));
      CU(batch_sweep(b->bd, b->NR, b->KT, b->NBmax, p, sw == ptfr - 1 && p == 1, true, b->bs));
    }
  if (ptfr == 0) CU(batch_sweep(b->bd, b->NR, b->KT, b->NBmax, 0, true, false, b->bs));
  CU(batch_energy_reduce(b->bd, b->bs));
  CU(batch_pt(b->bd, b->bs));
  return EA_OK;
}

static int batch_cycle(ea_batch *b, int ptfr) {
  if (!b->cycle || b->cycle_ptfr != ptfr) {
    if (b->cycle) { cudaGraphExecDestroy(b->cycle); b->cycle = nullptr; }
    cudaGraph_t graph = nullptr;
    CU(cudaStreamBeginCapture(b->bs, cudaStreamCaptureModeThreadLocal));
    const int rc = batch_cycle_launch(b, ptfr);
    const cudaError_t e = cudaStreamEndCapture(b->bs, &graph);
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    CU(e);
    const cudaError_t ei = cudaGraphInstantiate(&b->cycle, graph, 0);
    cudaGraphDestroy(graph);
    CU(ei);
    b->cycle_ptfr = ptfr;
  }
  CU(cudaGraphLaunch(b->cycle, b->bs));
  return EA_OK;
}

static int batch_houdayer(ea_batch *b, int nclust) {
  const int n = (int)b->jobs.size();
  int rc;
  for (ea_ctx *c : b->jobs)
    if ((rc = houdayer_prepare(c, nclust))) return rc;
  if ((rc = batch_upload(b))) return rc;
  for (ea_ctx *c : b->jobs) CU(cudaStreamWaitEvent(b->bs, c->drawn[c->cur], 0));
  CU(batch_pairs(b->bd, b->bs));
  UTable &u = b->u;
  for (int grp = 0; grp < 2; ++grp) {
    for (int i = 0; i < n; ++i) u.u[i] = b->jobs[i]->U[b->jobs[i]->cur][grp];
    CU(batch_houdayer_group(b->bd, u, grp, b->bs));
    // jobs whose planes exceed the slab labelling take the one-job path
    for (int i = 0; i < n; ++i) {
      const uint32_t *pre = b->up_pre.data() + (size_t)KB_SLAB * (n + 1);
      if (pre[i + 1] != pre[i]) continue;
      JobDev jg = b->jobs[i]->j;
      jg.U = u.u[i];
      CU(launch_houdayer_group(jg, grp, b->bs));
    }
  }
  for (ea_ctx *c : b->jobs)
    if ((rc = houdayer_finish(c, b->bs))) return rc;
  return EA_OK;
}

int ea_batch_run_bin(ea_batch *b, const ea_cadence *cad) {
  if (!b || !cad || cad->itmax < 1 || cad->houfr < 1 || cad->mesfr < 1 || cad->ptfr < 0)
    return fail(EA_ERR_ARG, "bad cadence");
  CU(cudaSetDevice(b->device));
  int frec, maxit;
  trw(cad->itmax, &frec, &maxit);
  // every job's earlier work comes first
  for (ea_ctx *c : b->jobs) {
    if (!c->have_temps) return fail(EA_ERR_STATE, "temperatures not set");
    if (cad->cluster && c->g.NR < 4) return fail(EA_ERR_ARG, "the Houdayer move needs at least 2 replicas per group");
    CU(cudaEventRecord(b->done, c->st));
    CU(cudaStreamWaitEvent(b->bs, b->done, 0));
  }
  // buffers that grow are reallocated only once the batch's earlier kernels ended
  // (a job that joined the batch since has none yet, so it costs no wait)
  bool grow = false;
  for (ea_ctx *c : b->jobs)
    grow = grow || (c->hist && maxit > c->hist_cap) ||
           (c->label && cad->cluster && norm_nclust(c->g, cad->nclust) > c->nclust_cap);
  if (grow) CU(cudaStreamSynchronize(b->bs));
  for (ea_ctx *c : b->jobs) {
    const Geometry &g = c->g;
    const size_t nsr = (size_t)g.ns * g.NR;
    if (maxit > c->hist_cap) {
      if (c->hist) cudaFree(c->hist);
      c->hist = nullptr;
      CU(dalloc(c->hist, nsr * maxit * g.NB));
      c->hist_cap = maxit;
    }
    c->j.hist = c->hist;
    c->j.maxit_trw = maxit;
    CU(cudaMemsetAsync(c->avgE, 0, nsr * g.NB * 8, b->bs));
    CU(cudaMemsetAsync(c->hist, 0, nsr * maxit * g.NB, b->bs));
    if (cad->cluster) {
      const int rc = ensure_cluster(c, norm_nclust(g, cad->nclust));
      if (rc) return rc;
    }
  }
  int rc = batch_upload(b);
  if (rc) return rc;
  for (int it = 0; it < cad->itmax; ++it) {
    for (int im = 0; im < cad->mesfr; ++im) {
      for (int ih = 0; ih < cad->houfr; ++ih) {
        // with ptfr = 0 the cycle measures the energies before the swaps
        // (measuring energies that are still fresh leaves them unchanged)
        if ((rc = batch_cycle(b, cad->ptfr))) return rc;
      }
      if (cad->cluster && (rc = batch_houdayer(b, cad->nclust))) return rc;
    }
    CU(batch_sweep(b->bd, b->NR, b->KT, b->NBmax, 0, true, false, b->bs));
    CU(batch_energy_reduce(b->bd, b->bs));
    CU(batch_measure(b->bd, (it % frec == frec - 1) ? it / frec : -1, b->bs));
  }
  // later work of each job comes after the batch
  CU(cudaEventRecord(b->done, b->bs));
  for (ea_ctx *c : b->jobs) {
    CU(cudaStreamWaitEvent(c->st, b->done, 0));
    c->energies_fresh = true;
  }
  return EA_OK;
}

int ea_batch_sync(ea_batch *b) {
  if (!b) return fail(EA_ERR_ARG, "null batch");
  CU(cudaSetDevice(b->device));
  CU(cudaStreamSynchronize(b->bs));
  return EA_OK;
}

int ea_batch_stream(ea_batch *b, void **stream) {
  if (!b || !stream) return fail(EA_ERR_ARG, "null argument");
  *stream = (void *)b->bs;
  return EA_OK;
}

int ea_init_run(ea_ctx *c, const uint64_t masters[4], const int32_t *list_samples, int64_t iter0, uint32_t jobid) {
  if (check(c) || !masters) return fail(EA_ERR_ARG, "null argument");
  const Geometry &g = c->g;
  std::vector<uint64_t> sJ(g.ns), su(g.ns), sMC(g.NR);
  int rc = ea_host_seeds(masters[0], masters[1], masters[2], masters[3], list_samples, g.ns, g.NR, sJ.data(),
                         su.data(), sMC.data());
  if (rc) return rc;
  std::vector<ea_generators> gen(1);
  std::vector<ea_hq> pt((size_t)g.ns * g.NR);
  if ((rc = ea_host_generators(sMC.data(), list_samples, g.ns, g.NR, masters[3], gen.data(), pt.data()))) return rc;
  if ((rc = ea_set_generators(c, gen.data(), pt.data()))) return rc;
  ea_geom eg;
  ea_get_geom(c, &eg);
  // the samples' spins and couplings are independent host streams: built
  // on up to 8 threads, then uploaded in sample order
  const size_t n = g.words_per_parity(), nj = (size_t)12 * g.half;
  std::vector<uint64_t> words((size_t)g.ns * (2 * n + nj));
  std::vector<int> rcs(g.ns, EA_OK);
  auto build = [&](int s) {
    uint64_t *w = words.data() + (size_t)s * (2 * n + nj);
    int32_t cnt = 0;
    rcs[s] = ea_host_init_spins(&eg, su[s], w, w + n);
    if (!rcs[s]) rcs[s] = ea_host_init_couplings(&eg, sJ[s], nullptr, w + 2 * n, &cnt);
  };
  const int nth = std::min(g.ns, 8);
  std::vector<std::thread> pool;
  for (int t = 0; t < nth; ++t)
    pool.emplace_back([&, t] {
      for (int s = t; s < g.ns; s += nth) build(s);
    });
  for (auto &t : pool) t.join();
  for (int s = 0; s < g.ns; ++s) {
    if (rcs[s]) return fail(rcs[s], "initial state of sample %d", s);
    const uint64_t *w = words.data() + (size_t)s * (2 * n + nj);
    if ((rc = ea_set_spins(c, s, w, w + n))) return rc;
    if ((rc = ea_set_couplings(c, s, w + 2 * n))) return rc;
  }
  if ((rc = ea_set_permutations(c, nullptr))) return rc;
  return ea_set_counter(c, iter0, jobid);
}

int ea_job_bytes(const ea_geom *gp, const ea_cadence *cad, const double *betas, uint64_t *bytes) {
  Geometry g;
  if (!gp || !bytes || !g.set(*gp)) return fail(EA_ERR_ARG, "geometry: L, Lz multiples of 8, 2<=NB<=255, 1<=nsamples<=32");
  // each allocation rounded to the allocator's granule: 2 MiB pages for
  // allocations of 1 MiB and more, 512 bytes below (small ones share pages)
  uint64_t tot = 0;
  auto add = [&](uint64_t n) {
    n = std::max<uint64_t>(n, 1);
    tot += n >= (1ull << 20) ? (n + (2ull << 20) - 1) & ~((2ull << 20) - 1) : (n + 511) & ~(uint64_t)511;
  };
  const uint64_t nsr = (uint64_t)g.ns * g.NR, NB = g.NB, half = g.half, V = g.V;
  const int ktmin = g.NR == 8 ? 1 : g.NR == 4 ? 2 : 4;
  add((uint64_t)g.ns * g.words_per_sample() * 8);            // spins
  add((uint64_t)g.ns * 12 * half * 8);                       // couplings
  add(12 * half * 4); add(2 * half);                         // neighbour table, flags
  add(NB * 256 * 8); add(NB * 256 * 2);                      // thresholds, pre-search
  add(nsr * NB); add(nsr * NB);                              // permutations
  add(g.NR * 16); add(g.NR * 4); add(g.NR * sizeof(ea_hq)); add(g.NR * sizeof(ea_xoshiro)); add(8);
  add(2 * ((half + ktmin - 1) / ktmin) * nsr * NB * 4);      // energy partials (two tile widths at most)
  add(nsr * NB * 4); add(nsr * sizeof(ea_hq)); add(NB * 8); add(NB * 4);
  for (int k = 0; k < 3; ++k) add(nsr * (NB - 1) * 8);       // tempering statistics
  add(8); add(sizeof(ea_hq)); add(16); add(nsr * NB * 8);    // inexact, random_c, pairs, averages
  uint64_t nexp = 0;                                         // glibc exp table
  if (betas) {
    std::vector<double> tab;
    std::vector<int32_t> off;
    pt_exp_table(betas, g.NB, tab, off);
    nexp = tab.size();
  } else {
    nexp = (NB - 1) * 25001;  // temperature steps down to 1e-3
  }
  add(nexp * 8);
  int maxit = 1;
  if (cad && cad->itmax > 0) {
    int frec;
    trw(cad->itmax, &frec, &maxit);
  }
  add(nsr * maxit * NB);                                     // temperature history
  if (cad && cad->cluster) {
    const uint64_t ncl = (uint64_t)norm_nclust(g, cad->nclust);
    for (int k = 0; k < 4; ++k) add(V * NB * g.ns * 8);      // uniforms: two sets of two groups
    add(V * ncl * g.ns * 4); add(V / 32 * ncl * g.ns * 4); add(2 * half * ncl * g.ns * 8);
    tot += 4ull << 20;                                       // cuRAND generator state
  }
  *bytes = tot + (4ull << 20);                               // streams, events, pages of the small allocations
  return EA_OK;
}

int ea_bin_results(ea_ctx *c, double *avgE, uint8_t *hist, int32_t *maxit_trw) {
  if (check(c)) return EA_ERR_ARG;
  if (set_device(c)) return EA_ERR_CUDA;
  const Geometry &g = c->g;
  const size_t nsr = (size_t)g.ns * g.NR;
  CU(cudaStreamSynchronize(c->st));
  const int maxit = c->j.maxit_trw;
  if (avgE) CU(cudaMemcpy(avgE, c->avgE, nsr * g.NB * 8, cudaMemcpyDeviceToHost));
  if (hist && c->hist) CU(cudaMemcpy(hist, c->hist, nsr * maxit * g.NB, cudaMemcpyDeviceToHost));
  if (maxit_trw) *maxit_trw = maxit;
  return ea_check_exact(c);
}

}  // extern "C"
