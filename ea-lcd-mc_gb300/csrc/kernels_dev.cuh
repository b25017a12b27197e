// kernels_dev.cuh -- device code of the hot path: helpers and the body of each
// kernel as a function of (job, block coordinates).  The one-job kernels
// (kernels.cu) and the persistent batched kernels (batch.cu) both call these
// bodies, so a job gives the same words alone and in a batch.
//
// The work is integer bit-slicing, so tensor cores play no part; the kernels
// are bound by the integer pipes (Philox + threshold search) and by HBM/L2
// traffic on the spin words.  Reference behaviour is cited per kernel (paths
// relative to the reference project).
#pragma once
#include "kernels.cuh"

namespace eagb {

typedef unsigned long long u64;

// ---------------------------------------------------------------------------
// Philox counter of a half-sweep (fill_bits.h:47-68): advance the replica's
// xoshiro256++ and Parisi-Rapuano generators once and place 52 entropy bits
// around the time counter and the job id.  One thread per replica.
// ---------------------------------------------------------------------------
__device__ __forceinline__ u64 d_rotl(u64 x, int k) { return (x << k) | (x >> (64 - k)); }

__device__ __forceinline__ u64 d_hq_next(ea_hq *h) {
  const uint8_t ip = h->ip, ip1 = h->ip1, ip2 = h->ip2, ip3 = h->ip3;
  const u64 a = h->ira[ip1] + h->ira[ip2];
  h->ira[ip] = a;
  h->PR = a ^ h->ira[ip3];
  h->zseed = h->zseed * 3202034522624059733ULL + 1;
  h->final = h->zseed + h->PR;
  h->ip = ip + 1; h->ip1 = ip1 + 1; h->ip2 = ip2 + 1; h->ip3 = ip3 + 1;
  return h->final;
}

// One step of a replica's two generators and the counter it gives for time
// counter `iter` (the state may live in global or shared memory).
__device__ __forceinline__ uint4 next_counter(ea_xoshiro *x, ea_hq *h, long long iter, int parity, uint32_t jobid) {
  u64 s0 = x->s[0], s1 = x->s[1], s2 = x->s[2], s3 = x->s[3];
  const u64 xf = d_rotl(s0 + s3, 23) + s0;
  const u64 t = s1 << 17;
  s2 ^= s0; s3 ^= s1; s1 ^= s2; s0 ^= s3; s2 ^= t; s3 = d_rotl(s3, 45);
  x->s[0] = s0; x->s[1] = s1; x->s[2] = s2; x->s[3] = s3; x->t = t; x->final = xf;
  const u64 pf = d_hq_next(h);
  u64 e = (pf + xf) >> 12;
  uint4 c;
  c.y = (uint32_t)((u64)iter >> 15);
  c.x = (uint32_t)((((u64)iter & 32767ULL) << 3) | ((u64)(parity & 1) << 2));
  c.x |= (uint32_t)((e & 0x3FFFULL) << 18); e >>= 14;
  c.y |= (uint32_t)((e & 0x7FULL) << 25); e >>= 7;
  c.z = (uint32_t)((e & 0x1FFFULL) << 19); e >>= 13;
  c.w = ((uint32_t)(e << 14)) | jobid;
  return c;
}

__device__ __forceinline__ void fill_bits_body(const JobDev &j, int parity) {
  const int r = threadIdx.x;
  const long long iter = *j.iter;
  __syncthreads();
  if (r < j.NR) j.ctr[r] = next_counter(j.xo + r, j.prc + r, iter, parity, j.jobid);
  if (r == 0) *j.iter = iter + 1;
}

// ---------------------------------------------------------------------------
// Random words: Philox4x32-10 (main.cu:996-1043), the post-mix of
// main.cu:1045-1060, and for each of the four 64-bit keys the first byte n with
// R < cum[n] (the heat-bath thresholds); this is the function the reference's
// pre-search + bisection computes (main.cu:1063-1078).  Here the pre-search is
// indexed by the top 8 bits so that every temperature's table fits in SMEM.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox10(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t k0,
                                         uint32_t k1) {
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    if (i) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const u64 p0 = (u64)0xD2511F53u * v0;
    const u64 p1 = (u64)0xCD9E8D57u * v2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ v1 ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ v3 ^ k1;
    v1 = (uint32_t)p1; v3 = (uint32_t)p0; v0 = n0; v2 = n2;
  }
}

// GCUM: the thresholds are read from global memory through the read-only
// cache instead of SMEM (the pre-search pins the byte without reading them
// for most R: 0.05-0.35 bisection steps per byte on the benchmark sets).
template <bool GCUM = false>
__device__ __forceinline__ uint32_t lut_byte(uint32_t hi, uint32_t lo, const u64 *cum, const uint16_t *pre) {
  const u64 R = ((u64)hi << 32) | lo;
  const uint32_t e = pre[hi >> 24];
  uint32_t a = e & 255u, b = e >> 8;
  while (a < b) {
    const uint32_t m = (a + b) >> 1;
    if (R < (GCUM ? __ldg(cum + m) : cum[m])) b = m; else a = m + 1;
  }
  return a;
}

// The same search with the 11-bit pre-search of presearch11 (host.cpp): a
// key in bucket t = hi >> 21 has its byte in [pre[t], pre[t+1]]; thresholds
// through the read-only cache.  Narrower buckets leave a bisection to fewer
// keys: 0.04 steps per byte on the benchmark sets against 0.18-0.21 with the
// 8-bit pre-search, and a warp waits for its slowest lane at each search.
__device__ __forceinline__ uint32_t lut_byte11(uint32_t hi, uint32_t lo, const u64 *cum, const uint8_t *pre) {
  const u64 R = ((u64)hi << 32) | lo;
  const uint32_t t = hi >> 21;
  uint32_t a = pre[t], b = pre[t + 1];
  while (a < b) {
    const uint32_t m = (a + b) >> 1;
    if (R < __ldg(cum + m)) b = m; else a = m + 1;
  }
  return a;
}

// One random word from a Philox counter: the four keys' bytes by `byte`
// (a threshold search), rotated as the post-mix says.
template <class Byte>
__device__ __forceinline__ uint32_t rnd_word_by(uint32_t cx, uint32_t cy, uint32_t cz, uint32_t cw, uint32_t key,
                                                uint32_t tid, Byte byte) {
  uint32_t v0 = cx, v1 = cy, v2 = cz, v3 = cw;
  philox10(v0, v1, v2, v3, tid, key);
  const uint32_t h = v0 ^ v2, l = v1 ^ v3;
  const uint32_t s0 = __funnelshift_l(v0, v1, 17) ^ h ^ __funnelshift_l(l, h, 21);
  const uint32_t s1 = __funnelshift_l(v1, v0, 17) ^ l ^ (l << 21);
  const uint32_t s2 = __funnelshift_l(l, h, 28);
  const uint32_t s3 = __funnelshift_l(h, l, 28);
  const uint32_t rot = (s0 + v1 + s2 + v3) >> 27;
  const uint32_t bb = byte(v0, s0) | (byte(v1, s1) << 8) | (byte(v2, s2) << 16) | (byte(v3, s3) << 24);
  return __funnelshift_l(bb, bb, rot);  // rotate left; rot 0 leaves the word as it is
}

template <bool GCUM = false>
__device__ __forceinline__ uint32_t rnd_word(uint32_t cx, uint32_t cy, uint32_t cz, uint32_t cw, uint32_t key,
                                             uint32_t tid, const u64 *cum, const uint16_t *pre) {
  return rnd_word_by(cx, cy, cz, cw, key, tid,
                     [&](uint32_t hi, uint32_t lo) { return lut_byte<GCUM>(hi, lo, cum, pre); });
}

// ---------------------------------------------------------------------------
// Multispin neighbour words: bit rotation across the sub-block wrap
// (main.cu:1154-1190) and the OBC fake bond patch (main.cu:1460-1472).
// ---------------------------------------------------------------------------
__device__ __forceinline__ u64 rot_dir(int d, u64 o) {
  switch (d) {
    case 0: return (o & 0x1111111111111111ull) << 3 | (o & ~0x1111111111111111ull) >> 1;
    case 1: return (o & 0x000F000F000F000Full) << 12 | (o & ~0x000F000F000F000Full) >> 4;
    case 2: return (o & 0x000000000000FFFFull) << 48 | (o & ~0x000000000000FFFFull) >> 16;
    case 3: return (o & 0x8888888888888888ull) >> 3 | (o & ~0x8888888888888888ull) << 1;
    case 4: return (o & 0xF000F000F000F000ull) >> 12 | (o & ~0xF000F000F000F000ull) << 4;
    default: return (o & 0xFFFF000000000000ull) >> 48 | (o & ~0xFFFF000000000000ull) << 16;
  }
}
#define MASK_TOP (~0xFFFF000000000000ull)  // keeps bz < 3 (main.cu:1207)
#define MASK_BOT (~0x000000000000FFFFull)  // keeps bz > 0 (main.cu:1206)

__device__ __forceinline__ void gather6(const u64 *oth, const int *nb, int flags, int parity, bool obc, int NR,
                                        u64 n[6]) {
#pragma unroll
  for (int d = 0; d < 6; ++d) {
    u64 w = oth[(size_t)nb[d] * NR];
    if ((flags >> d) & 1) w = rot_dir(d, w);
    n[d] = w;
  }
  if (obc) {
    const u64 aux = parity == 0 ? n[1] : n[4];
    if (flags & 0x40) n[2] = (n[2] & MASK_TOP) | (aux & ~MASK_TOP);
    if (flags & 0x80) n[5] = (n[5] & MASK_BOT) | (aux & ~MASK_BOT);
  }
}

// Bit-sliced local field and Metropolis flip mask (main.cu:1474-1506): flip with
// probability min(1, p^(3-c)) where c counts satisfied-minus-unsatisfied pairs.
__device__ __forceinline__ u64 flip_mask(const u64 f[6], u64 b0, u64 b1, u64 b2) {
  u64 k1 = f[0] ^ f[1], k2 = f[0] & f[1];
  const u64 j1 = k1 ^ f[2], j2 = k2 ^ (k1 & f[2]);
  k1 = f[3] ^ f[4]; k2 = f[3] & f[4];
  const u64 j3 = k1 ^ f[5], j4 = k2 ^ (k1 & f[5]);
  b1 = b0 & b1; b2 = b1 & b2;
  const u64 id2 = b1, id1 = (b0 ^ b1) | b2, j24 = j2 | j4;
  return (j1 & j3 & id1) | ((j24 | id2) & (j1 | j3 | id1)) | ((j2 & j4) | (j24 & id2));
}

// ---------------------------------------------------------------------------
// Fused half-sweep.  A CTA owns KT half-sites of one parity.  It stages every
// temperature's 8-bit pre-search (NB x 512 B) in SMEM -- the thresholds
// themselves, rarely needed past the pre-search, are read through the
// read-only cache, which keeps a CTA's SMEM small -- generates the 3 random words
// of each (beta, half-site, replica) once -- they are shared by all samples, as
// the reference's random buffer has no sample axis (main.cu:1430) -- and then
// updates every (sample, clone, half-site, replica) word of its tile, picking
// the words of the clone's current temperature.  The random word indices
// depend only on (beta, half-site, replica, counter), never on the launch
// shape.  With ENERGY it also adds up, per (sample, clone, replica), the
// energy of the updated words (each bond has exactly one end on each parity).
// ---------------------------------------------------------------------------
template <int NR, int KT, bool UPDATE>
// stage = false: the thresholds of this job are already in SMEM (the block's
// previous tile was of the same job).
__device__ __forceinline__ void sweep_body(const JobDev &j, int tile, int parity, int energy, unsigned char *smem,
                                           bool stage = true) {
  const int NB = j.NB, half = j.half;
  u64 *s_rnd = reinterpret_cast<u64 *>(smem);
  uint16_t *s_pre = reinterpret_cast<uint16_t *>(s_rnd + (UPDATE ? 3 * NB * KT * NR : 0));
  int *s_nb = reinterpret_cast<int *>(s_pre + (UPDATE ? NB * 256 : 0));
  const int k0 = tile * KT;
  const int tid = threadIdx.x, nth = blockDim.x;

  if (UPDATE && stage) {
    const uint4 *ps = reinterpret_cast<const uint4 *>(j.pre);
    uint4 *pd = reinterpret_cast<uint4 *>(s_pre);
    for (int i = tid; i < NB * 32; i += nth) pd[i] = ps[i];
  }
  if (tid < KT * 8) {
    const int kk = tid >> 3, f = tid & 7, k = k0 + kk;
    int v = 0;
    if (k < half) v = f < 6 ? j.nbidx[(parity * 6 + f) * half + k] : (f == 6 ? (int)j.nbflag[parity * half + k] : 0);
    s_nb[tid] = v;
  }
  __syncthreads();

  if (UPDATE) {
    const int ntrip = NB * KT * NR;
    for (int t = tid; t < ntrip; t += nth) {
      const int r = t % NR, kk = (t / NR) % KT, b = t / (NR * KT), k = k0 + kk;
      if (k >= half) continue;
      const uint32_t tp = (uint32_t)((b * half + k) * NR + r);
      const uint4 c = j.ctr[r];
      const uint32_t key = j.keys[r];
      const u64 *cum = j.cum + b * 256;
      const uint16_t *pre = s_pre + b * 256;
      uint32_t w[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) w[q] = rnd_word<true>(c.x + q, c.y, c.z + tp, c.w, key, tp, cum, pre);
      const int o = (b * KT + kk) * NR + r, plane = NB * KT * NR;
      s_rnd[o] = ((u64)w[0] << 32) | w[1];
      s_rnd[plane + o] = ((u64)w[2] << 32) | w[3];
      s_rnd[2 * plane + o] = ((u64)w[4] << 32) | w[5];
    }
    __syncthreads();
  }

  // Update phase.  Lanes form groups of G = KT*NR; a lane keeps its
  // (half-site, replica) and its neighbour record for the whole loop, and a
  // group walks a contiguous run of (sample, clone) pairs, clone fastest, so
  // the G lanes of a group touch G consecutive words of one clone array and a
  // lane loads the six coupling words of its (sample, half-site) once per
  // sample rather than once per word.
  constexpr int G = KT * NR;
  const size_t wpc = (size_t)half * NR, wpp = wpc * NB;
  const int lg = tid % G, grp = tid / G, ngrp = nth / G;
  const int r = lg % NR, kk = lg / NR, k = k0 + kk;
  const bool kvalid = k < half;
  const bool obc = j.bc != EA_PBC;
  int nb[6];
#pragma unroll
  for (int d = 0; d < 6; ++d) nb[d] = s_nb[kk * 8 + d];
  const int nflags = s_nb[kk * 8 + 6];
  const int nsc = j.ns * NB, iters = (nsc + ngrp - 1) / ngrp;
  const int sc0 = grp * iters;
  int s = sc0 / NB, c = sc0 - s * NB, js = -1;
  u64 jw[6];
  for (int it = 0, sc = sc0; it < iters; ++it, ++sc) {
    const bool valid = kvalid && sc < nsc;
    int e = 0;
    if (valid) {
      u64 *base = j.spins + (size_t)s * 2 * wpp + (size_t)c * wpc;
      u64 *tgt = base + (size_t)parity * wpp + (size_t)k * NR + r;
      const u64 *oth = base + (size_t)(1 - parity) * wpp + r;
      if (s != js) {
        const u64 *Jp = j.J + ((size_t)s * 2 + parity) * 6 * half + k;
#pragma unroll
        for (int d = 0; d < 6; ++d) jw[d] = __ldg(Jp + (size_t)d * half);
        js = s;
      }
      const u64 sv = *tgt;
      u64 n[6];
      gather6(oth, nb, nflags, parity, obc, NR, n);
      u64 f[6];
#pragma unroll
      for (int d = 0; d < 6; ++d) f[d] = sv ^ jw[d] ^ n[d];
      u64 fl = 0;
      if (UPDATE) {
        const int beta = j.wbtc[(s * NR + r) * NB + c];
        const int o = (beta * KT + kk) * NR + r, plane = NB * KT * NR;
        fl = flip_mask(f, s_rnd[o], s_rnd[plane + o], s_rnd[2 * plane + o]);
        *tgt = sv ^ fl;
      }
      if (energy) {
        int le = 0;
#pragma unroll
        for (int d = 0; d < 6; ++d) le += __popcll(f[d] ^ fl);
        e = 6 * 64 - 2 * le;
      }
    }
    if (energy) {
#pragma unroll
      for (int m = NR; m < G; m <<= 1) e += __shfl_xor_sync(0xffffffffu, e, m);
      if (valid && kk == 0) j.epart[(((size_t)tile * j.ns + s) * NB + c) * NR + r] = e;
    }
    if (++c == NB) { c = 0; ++s; }
  }
}

// E[s][rep][clone] = sum over tiles (thread per (s, clone, rep)).
__device__ __forceinline__ void energy_reduce_body(const JobDev &j, int i) {
  const int n = j.ns * j.NB * j.NR;
  if (i >= n) return;
  int e = 0;
  for (int t = 0; t < j.ntiles; ++t) e += j.epart[(size_t)t * n + i];
  const int r = i % j.NR, c = (i / j.NR) % j.NB, s = i / (j.NR * j.NB);
  j.E[((size_t)s * j.NR + r) * j.NB + c] = e;
}

// ---------------------------------------------------------------------------
// Parallel tempering (upd.c:3-48), one warp per (sample, replica) chain: the
// warp stages the PT generator's lag table in SMEM, lane 0 walks the NB-1
// pairs in order with FP64 arithmetic rounded as on the host, and exp(pt) comes
// from the host's libm through the table built at set-up.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pt_body(const JobDev &j, int s, int ry, u64 (*s_ira)[256], uint8_t (*s_wc)[256]) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = ry * 8 + w;
  if (r >= j.NR) return;
  const int NB = j.NB;
  const size_t o = (size_t)s * j.NR + r;
  ea_hq *h = j.pt + o;
  for (int i = lane; i < 256; i += 32) s_ira[w][i] = h->ira[i];
  for (int i = lane; i < NB; i += 32) s_wc[w][i] = j.wctb[o * NB + i];
  __syncwarp();
  if (lane == 0) {
    u64 *ira = s_ira[w];
    uint8_t *wc = s_wc[w];
    uint8_t ip = h->ip, ip1 = h->ip1, ip2 = h->ip2, ip3 = h->ip3;
    u64 zseed = h->zseed, PR = h->PR, fin = h->final;
    const int32_t *E = j.E + o * NB;
    double *acc = j.acc + o * (NB - 1), *att = j.att + o * (NB - 1), *accraw = j.accraw + o * (NB - 1);
    const double FNORM = 5.4210108624275218e-20;
    for (int i = 0; i < NB - 1; ++i) {
      att[i] += 1.0;
      const int dE = E[wc[i + 1]] - E[wc[i]];
      const double pt = __dmul_rn(-__dsub_rn(j.betas[i + 1], j.betas[i]), (double)dE);
      const u64 a = ira[ip1] + ira[ip2];
      ira[ip] = a;
      PR = a ^ ira[ip3];
      zseed = zseed * 3202034522624059733ULL + 1;
      fin = zseed + PR;
      ++ip; ++ip1; ++ip2; ++ip3;
      bool change;
      if (pt >= 0.0) {
        acc[i] += 1.0;
        change = true;
      } else {
        const int base = j.expoff[i], n = j.expoff[i + 1] - base, m = (-dE) >> 1;
        double ex;
        if (!(dE & 1) && m >= 1 && m <= n) {
          ex = j.exptab[base + m - 1];
        } else {
          ex = exp(pt);  // exp(pt) < 2^-72 here: decides only when the draw is 0
          if (fin == 0 || (dE & 1)) atomicAdd(j.inexact, 1ULL);
        }
        acc[i] += ex;
        change = __dmul_rn(FNORM, __ull2double_rn(fin)) < ex;
      }
      if (change) {
        const uint8_t t = wc[i]; wc[i] = wc[i + 1]; wc[i + 1] = t;
        accraw[i] += 1.0;
      }
    }
    h->ip = ip; h->ip1 = ip1; h->ip2 = ip2; h->ip3 = ip3;
    h->zseed = zseed; h->PR = PR; h->final = fin;
  }
  __syncwarp();
  for (int i = lane; i < 256; i += 32) h->ira[i] = s_ira[w][i];
  for (int i = lane; i < NB; i += 32) {
    const uint8_t c = s_wc[w][i];
    j.wctb[o * NB + i] = c;
    j.wbtc[o * NB + c] = (uint8_t)i;
  }
}

// Energy average in beta order and temperature history (main.cu:208-228).
__device__ __forceinline__ void measure_body(const JobDev &j, int i, int itm) {
  const int n = j.ns * j.NR * j.NB;
  if (i >= n) return;
  const size_t o = i / j.NB;
  const int b = i % j.NB;
  j.avgE[i] += (double)j.E[o * j.NB + j.wctb[o * j.NB + b]];
  if (itm >= 0) j.hist[(o * j.maxit_trw + itm) * j.NB + b] = j.wbtc[o * j.NB + b];
}

// ---------------------------------------------------------------------------
// Houdayer move.
// ---------------------------------------------------------------------------
// Replica pairs of both groups with random_c (main.cu:409-421).
__device__ __forceinline__ void pairs_body(const JobDev &j) {
  const int h = j.NR / 2;
  for (int g = 0; g < 2; ++g) {
    int idx[32];
    for (int k = 0; k < h; ++k) idx[k] = k + g * h;
    for (int k = 0; k < h - 1; ++k) {
      const u64 f = d_hq_next(j.rc);
      const int q = k + (int)(((uint32_t)(f >> 32)) % (uint32_t)(h - k));
      const int t = idx[k]; idx[k] = idx[q]; idx[q] = t;
    }
    j.pairs[2 * g] = idx[0];
    j.pairs[2 * g + 1] = idx[1];
  }
}

// q = s_r1 ^ s_r2 per (sample, beta < nclust, parity, half) (main.cu:889-936).
__device__ __forceinline__ void overlap_body(const JobDev &j, int g, int w, size_t lat) {
  if (w >= 2 * j.half) return;
  const size_t i = lat * 2 * j.half + w;
  const int p = w >= j.half, k = w - p * j.half;
  const int s = j.fd_nclust.div((uint32_t)lat), b = (int)lat - s * j.nclust;
  const int r1 = j.pairs[2 * g], r2 = j.pairs[2 * g + 1];
  const int c1 = j.wctb[((size_t)s * j.NR + r1) * j.NB + b], c2 = j.wctb[((size_t)s * j.NR + r2) * j.NB + b];
  const size_t wpc = (size_t)j.half * j.NR, wpp = wpc * j.NB;
  const u64 *base = j.spins + (size_t)s * 2 * wpp + (size_t)p * wpp + (size_t)k * j.NR;
  j.Q[i] = base[(size_t)c1 * wpc + r1] ^ base[(size_t)c2 * wpc + r2];
}

// Overlap bit of a site in natural order (x + L y + L^2 z): parity, half index
// and bit of the multispin word (ini.c:355-375).
__device__ __forceinline__ int q_bit(const JobDev &j, const u64 *Q, int x, int y, int z) {
  const int bx = j.fd_ml.div(x), gx = x - bx * j.msc_l, by = j.fd_ml.div(y), gy = y - by * j.msc_l;
  const int bz = j.fd_mlz.div(z), gz = z - bz * j.msc_lz;
  const int m = gx + j.msc_l * gy + j.msc_s * gz, p = (x ^ y ^ z) & 1;
  return (int)((Q[(size_t)p * j.half + (m >> 1)] >> (bx + 4 * by + 16 * bz)) & 1);
}

__device__ __forceinline__ uint32_t cc_find(const uint32_t *lab, uint32_t i) {
  uint32_t l = lab[i];
  while (l != i) { i = l; l = lab[i]; }
  return l;
}

// Lock-free union: the larger of the two roots is hung below the smaller one
// with atomicMin; when another thread got there first the walk continues from
// the value it left.  Labels only decrease, so every chain ends at the
// smallest index of its cluster.  Works on global and shared memory.
__device__ __forceinline__ void cc_unite(uint32_t *lab, uint32_t a, uint32_t b) {
  uint32_t l1 = cc_find(lab, a), l2 = cc_find(lab, b);
  if (l1 == l2) return;
  if (l1 < l2) { const uint32_t t = l1; l1 = l2; l2 = t; }
  for (;;) {
    const uint32_t l3 = atomicMin(&lab[l1], l2);
    if (l3 == l2 || l3 == l1) return;  // already joined, or l1 was a root and now hangs below l2
    if (l3 > l2) { l1 = l3; }
    else { l1 = l2; l2 = l3; }
  }
}

// Slab labelling.  A CTA labels the equal-overlap clusters of D consecutive z
// planes of one (sample, beta) lattice in SMEM.  Local index order is natural
// order shifted by z0 L^2, so a slab root is the smallest global index of its
// slab piece; only bonds between slabs are left for k_cc_merge.

// Planes of up to 1024 sites: one thread per (x, y) column and P planes
// (at most 16 sites a thread), in lock-step rounds so that no lane walks a
// long chain while the others wait:
//   hook:  every bond whose two labels differ hangs the larger label below
//          the smaller (atomicMin);
//   jump:  lab[i] = lab[lab[i]] until every label is a root;
// until a hook round finds nothing to do.  Labels only decrease and always
// name a site of the same cluster, so at the end every site holds the
// smallest index of its slab cluster.  The bonds are those of the union-find
// of the reference (HoudayerXEA.cu:77-121): -x and -y periodic, -z inside the
// slab.

// Threads from S*P on (a batched launch sized for a larger plane) own no
// sites and only take part in the barriers.
__device__ __forceinline__ void cc_slab_body(const JobDev &j, int D, int P, int slab, size_t lat, uint32_t *lab, uint8_t *qs) {
  const int L = j.L, S = L * L, t = threadIdx.x;
  const int z0 = slab * D, nz = t < S * P ? min(D, j.Lz - z0) : 0;
  const u64 *Q = j.Q + lat * 2 * j.half;
  const int zp = j.fd_S.div(t), xy = t - zp * S, y = j.fd_L.div(xy), x = xy - y * L;
  {
    const int bx = j.fd_ml.div(x), by = j.fd_ml.div(y);
    const int mxy = (x - bx * j.msc_l) + j.msc_l * (y - by * j.msc_l), sxy = bx + 4 * by;
    int z = z0 + zp, bz = j.fd_mlz.div(z), gz = z - bz * j.msc_lz;
    for (int zl = zp; zl < nz; zl += P) {
      const int i = xy + S * zl, m = mxy + j.msc_s * gz, p = (x ^ y ^ z) & 1;
      qs[i] = (uint8_t)((Q[(size_t)p * j.half + (m >> 1)] >> (sxy + 16 * bz)) & 1);
      lab[i] = (uint32_t)i;
      z += P;
      gz += P;
      while (gz >= j.msc_lz) { gz -= j.msc_lz; ++bz; }
    }
  }
  __syncthreads();
  const int xm = x == 0 ? L - 1 : x - 1, ym = y == 0 ? L - 1 : y - 1;
  const int ixm = xm + L * y, iym = x + L * ym;
  // bond bits of this thread's sites: 3 per site (-x, -y, -z)
  u64 bonds = 0;
  {
    int k = 0;
    for (int zl = zp; zl < nz; zl += P, ++k) {
      const int i = xy + S * zl, q = qs[i], pl = S * zl;
      // site 0 tests its x-wrap bond against x = cc_xq (see JobDev::cc_xq)
      const int xt = (z0 == 0 && i == 0) ? j.cc_xq : xm;
      const u64 b = (u64)(qs[xt + L * y + pl] == q) | ((u64)(qs[iym + pl] == q) << 1) |
                    ((u64)(zl > 0 && qs[i - S] == q) << 2);
      bonds |= b << (3 * k);
    }
  }
  for (;;) {
    int hooked = 0;
    {
      int k = 0;
      for (int zl = zp; zl < nz; zl += P, ++k) {
        const unsigned b = (unsigned)(bonds >> (3 * k)) & 7u;
        if (!b) continue;
        const int i = xy + S * zl, pl = S * zl;
        const uint32_t li = lab[i];
        if (b & 1) {
          const uint32_t lj = lab[ixm + pl];
          if (lj != li) { atomicMin(&lab[max(li, lj)], min(li, lj)); hooked = 1; }
        }
        if (b & 2) {
          const uint32_t lj = lab[iym + pl];
          if (lj != li) { atomicMin(&lab[max(li, lj)], min(li, lj)); hooked = 1; }
        }
        if (b & 4) {
          const uint32_t lj = lab[i - S];
          if (lj != li) { atomicMin(&lab[max(li, lj)], min(li, lj)); hooked = 1; }
        }
      }
    }
    if (!__syncthreads_or(hooked)) break;
    for (;;) {
      int moved = 0;
      for (int zl = zp; zl < nz; zl += P) {
        const int i = xy + S * zl;
        const uint32_t l = lab[i], ll = lab[l];
        if (ll != l) { lab[i] = ll; moved = 1; }
      }
      if (!__syncthreads_or(moved)) break;
    }
  }
  uint32_t *glab = j.label + lat * j.V + (size_t)z0 * S;
  const uint32_t off = (uint32_t)z0 * S;
  for (int zl = zp; zl < nz; zl += P) glab[xy + S * zl] = off + lab[xy + S * zl];
}

// Bonds across slab faces (z = f D with z - 1), and the z wrap under PBC,
// merged into the global labels.
__device__ __forceinline__ void cc_merge_body(const JobDev &j, int D, int nslab, int r, size_t lat) {
  const int L = j.L, S = L * L;
  if (r >= nslab * S) return;
  const int f = j.fd_S.div(r), xy = r - f * S;
  int z, zm;
  if (f == 0) {
    if (j.bc != EA_PBC) return;
    z = 0; zm = j.Lz - 1;
  } else {
    z = f * D; zm = z - 1;
  }
  const int y = j.fd_L.div(xy), x = xy - y * L;
  const u64 *Q = j.Q + lat * 2 * j.half;
  if (q_bit(j, Q, x, y, z) == q_bit(j, Q, x, y, zm))
    cc_unite(j.label + lat * j.V, (uint32_t)(xy + S * z), (uint32_t)(xy + S * zm));
}

// After the merge, every slab root whose piece was joined across a face is
// re-pointed straight at its cluster's root; all such pieces touch a face, so
// walking once from each face site reaches them.  Afterwards any site finds
// its root in at most three loads (site -> slab root -> root).  Plain stores:
// every value written is the final root of the same cluster.
__device__ __forceinline__ void cc_compress_body(const JobDev &j, int D, int nslab, int r, size_t lat) {
  const int L = j.L, S = L * L;
  if (r >= nslab * S) return;
  const int f = j.fd_S.div(r), xy = r - f * S;
  int z, zm;
  if (f == 0) {
    if (j.bc != EA_PBC) return;
    z = 0; zm = j.Lz - 1;
  } else {
    z = f * D; zm = z - 1;
  }
  uint32_t *lab = j.label + lat * j.V;
  const uint32_t a = lab[xy + S * z], b = lab[xy + S * zm];
  const uint32_t ra = cc_find(lab, a), rb = cc_find(lab, b);
  if (ra != a) lab[a] = ra;
  if (rb != b) lab[b] = rb;
}

// Offsets, in natural site index, of the 64 sites of a multispin word from
// its bit-0 site: bit = bx + 4 by + 16 bz.
__device__ __forceinline__ int word_bit_offset(const JobDev &j, int bit) {
  return (bit & 3) * j.msc_l + ((bit >> 2) & 3) * j.msc_l * j.L + (bit >> 4) * j.msc_lz * j.L * j.L;
}

// Natural index of the bit-0 site of word (p, k).
__device__ __forceinline__ int word_site0(const JobDev &j, int p, int k) {
  const int hl = j.msc_l >> 1;
  const int row = j.fd_hl.div(k), gz = j.fd_ml.div(row), gy = row - gz * j.msc_l;
  const int gx = 2 * (k - row * hl) + ((gy + gz + p) & 1);
  return gx + j.L * gy + j.L * j.L * gz;
}

// Selection and flip of one lattice in one CTA (HoudayerXEA.cu:54-75,358-374;
// main.cu:776-832,938-991): bit i of s_bits is [U(root(i)) < 0.5], built in
// natural order (coalesced label reads, one ballot per 32 sites); then each
// word gathers its 64 bits from SMEM, q' = q xor sel, and s_r1 ^= q',
// s_r2 ^= q'.  s_bits holds V/32 words, s_off 64.
__device__ __forceinline__ void flip_body(const JobDev &j, const double *U, int g, size_t lat, uint32_t *s_bits,
                                          int *s_off) {
  const int t = threadIdx.x, nth = blockDim.x;
  const int s = j.fd_nclust.div((uint32_t)lat), b = (int)lat - s * j.nclust;
  const uint32_t *lab = j.label + lat * j.V;
  const double *u = U + ((size_t)s * j.NB + b) * j.V;
  if (t < 64) s_off[t] = word_bit_offset(j, t);
  for (int base = 0; base < j.V; base += nth) {
    const int site = base + t;
    bool sel = false;
    if (site < j.V) sel = __ldg(u + cc_find(lab, (uint32_t)site)) < 0.5;
    const unsigned ball = __ballot_sync(0xffffffffu, sel);
    if ((t & 31) == 0 && site < j.V) s_bits[site >> 5] = ball;
  }
  __syncthreads();
  const int r1 = j.pairs[2 * g], r2 = j.pairs[2 * g + 1];
  const int c1 = j.wctb[((size_t)s * j.NR + r1) * j.NB + b], c2 = j.wctb[((size_t)s * j.NR + r2) * j.NB + b];
  const size_t wpc = (size_t)j.half * j.NR, wpp = wpc * j.NB;
  const u64 *Q = j.Q + lat * 2 * j.half;
  for (int w = t; w < 2 * j.half; w += nth) {
    const int p = w >= j.half, k = w - p * j.half;
    const int s0 = word_site0(j, p, k);
    u64 mask = 0;
#pragma unroll 16
    for (int bit = 0; bit < 64; ++bit) {
      const int site = s0 + s_off[bit];
      mask |= (u64)((s_bits[site >> 5] >> (site & 31)) & 1u) << bit;
    }
    const u64 qn = Q[w] ^ mask;
    u64 *base = j.spins + (size_t)s * 2 * wpp + (size_t)p * wpp + (size_t)k * j.NR;
    base[(size_t)c1 * wpc + r1] ^= qn;
    base[(size_t)c2 * wpc + r2] ^= qn;
  }
}

// Cluster selection, natural order: bit i of sel[lat][i / 32] is
// [U(root(i)) < 0.5] for site i (HoudayerXEA.cu:358-374).  Consecutive lanes
// take consecutive sites, so the label reads are coalesced; the decisions of
// a lattice (V / 8 bytes) then stay in cache for the word-order flip.
__device__ __forceinline__ void select_body(const JobDev &j, const double *U, int site, size_t lat) {
  const int s = j.fd_nclust.div((uint32_t)lat), b = (int)lat - s * j.nclust;
  bool sel = false;
  if (site < j.V) {
    const uint32_t root = cc_find(j.label + lat * j.V, (uint32_t)site);
    sel = __ldg(U + ((size_t)s * j.NB + b) * j.V + root) < 0.5;
  }
  const unsigned ball = __ballot_sync(0xffffffffu, sel);
  if ((threadIdx.x & 31) == 0 && site < j.V) j.sel[lat * (j.V >> 5) + (site >> 5)] = ball;
}

// q' = q xor [selected] packed back into words, then s_r1 ^= q', s_r2 ^= q'
// (HoudayerXEA.cu:54-75; main.cu:776-832,938-991).  Two warps per word, one
// lane per bit.
__device__ __forceinline__ void apply_body(const JobDev &j, int g, int bx, size_t lat, unsigned *s_sel) {
  const int t = threadIdx.x, wl = t >> 6, bit = t & 63;
  const int w = bx * 4 + wl;            // word of this lattice: parity * half + k
  const size_t i = lat * 2 * j.half + w;
  const bool valid = w < 2 * j.half;
  const int p = w >= j.half, k = w - p * j.half;
  const int s = j.fd_nclust.div((uint32_t)lat), b = (int)lat - s * j.nclust;
  bool sel = false;
  if (valid) {
    const int hl = j.msc_l >> 1;
    const int row = j.fd_hl.div(k), gz = j.fd_ml.div(row), gy = row - gz * j.msc_l;
    const int gx = 2 * (k - row * hl) + ((gy + gz + p) & 1);
    const int x = gx + (bit & 3) * j.msc_l, y = gy + ((bit >> 2) & 3) * j.msc_l, z = gz + (bit >> 4) * j.msc_lz;
    const uint32_t site = (uint32_t)(x + j.L * y + j.L * j.L * z);
    sel = (__ldg(j.sel + lat * (j.V >> 5) + (site >> 5)) >> (site & 31)) & 1u;
  }
  const unsigned ball = __ballot_sync(0xffffffffu, sel);
  if ((t & 31) == 0) s_sel[t >> 5] = ball;
  __syncthreads();
  if (!valid || bit != 0) return;
  const u64 qn = j.Q[i] ^ ((u64)s_sel[2 * wl] | ((u64)s_sel[2 * wl + 1] << 32));
  const int r1 = j.pairs[2 * g], r2 = j.pairs[2 * g + 1];
  const int c1 = j.wctb[((size_t)s * j.NR + r1) * j.NB + b], c2 = j.wctb[((size_t)s * j.NR + r2) * j.NB + b];
  const size_t wpc = (size_t)j.half * j.NR, wpp = wpc * j.NB;
  u64 *base = j.spins + (size_t)s * 2 * wpp + (size_t)p * wpp + (size_t)k * j.NR;
  base[(size_t)c1 * wpc + r1] ^= qn;
  base[(size_t)c2 * wpc + r2] ^= qn;
}

}  // namespace eagb
