// sp.cu -- kernels of the sample-packed layout (64 samples per word) and its
// C ABI (ea_sp_*).  See sp.cuh for the layout.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "host.hpp"
#include "kernels_dev.cuh"
#include "sp.cuh"

namespace eagb {

void set_last_error(const char *msg);  // api.cu

// ---------------------------------------------------------------------------
// Philox counters of a colour pass: the reference's fill_bits step per
// replica (fill_bits.h:47-68) with the pass counter in place of the
// half-sweep counter (its parity bit = the counter's lowest bit, as for
// half-sweeps), so every pass of every sweep has its own counters.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sp_fill_body(const SpDev &d) {
  JobDev j{};
  j.NR = d.NR; j.xo = d.xo; j.prc = d.prc; j.ctr = d.ctr; j.iter = d.iter; j.jobid = d.jobid;
  const int parity = (int)(*d.iter & 1);
  fill_bits_body(j, parity);
}

// ---------------------------------------------------------------------------
// One colour pass.  A CTA owns kt sites of the colour: it stages every
// temperature's thresholds in SMEM, draws the three random words of each
// (slot, site, replica) once -- shared by the nw sample words, as the
// reference shares them across samples (main.cu:1430) -- and updates all
// (word, site, replica, slot) words of its tile in memory order, so that
// consecutive lanes touch consecutive words of a site.  The Philox thread
// index of (slot b, site i, replica r) is (b*V + i)*NR + r.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sp_pass_body(const SpDev &d, int off, int n, int tile, unsigned char *smem) {
  const int NB = d.NB, NR = d.NR, kt = d.kt, V = d.V;
  u64 *s_cum = reinterpret_cast<u64 *>(smem);
  uint16_t *s_pre = reinterpret_cast<uint16_t *>(s_cum + NB * 256);
  u64 *s_rnd = reinterpret_cast<u64 *>(s_pre + NB * 256);
  int *s_nb = reinterpret_cast<int *>(s_rnd + 3 * NB * kt * NR);  // [kt][7]: site, 6 neighbours
  const int tid = threadIdx.x, nth = blockDim.x;
  const int k0 = tile * kt;
  {
    const uint4 *cs = reinterpret_cast<const uint4 *>(d.cum);
    uint4 *cd = reinterpret_cast<uint4 *>(s_cum);
    for (int i = tid; i < NB * 128; i += nth) cd[i] = cs[i];
    const uint4 *ps = reinterpret_cast<const uint4 *>(d.pre);
    uint4 *pd = reinterpret_cast<uint4 *>(s_pre);
    for (int i = tid; i < NB * 32; i += nth) pd[i] = ps[i];
  }
  for (int i = tid; i < kt * 7; i += nth) {
    const int kk = i / 7, f = i % 7, k = k0 + kk;
    int v = -1;
    if (k < n) {
      const int site = d.col_sites[off + k];
      v = f == 0 ? site : d.nb[(size_t)site * 6 + f - 1];
    }
    s_nb[i] = v;
  }
  __syncthreads();
  // random words at [site of the tile][replica][slot]: the update phase's
  // consecutive lanes (consecutive slots) then read consecutive words
  const int plane = NB * kt * NR;
  for (int t = tid; t < plane; t += nth) {
    const int b = t % NB, r = (t / NB) % NR, kk = t / (NB * NR);
    if (k0 + kk >= n) continue;
    const int site = s_nb[kk * 7];
    const uint32_t tp = (uint32_t)(((size_t)b * V + site) * NR + r);
    const uint4 c = d.ctr[r];
    const uint32_t key = d.keys[r];
    const u64 *cum = s_cum + b * 256;
    const uint16_t *pre = s_pre + b * 256;
    uint32_t w[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) w[q] = rnd_word(c.x + q, c.y, c.z + tp, c.w, key, tp, cum, pre);
    s_rnd[t] = ((u64)w[0] << 32) | w[1];
    s_rnd[plane + t] = ((u64)w[2] << 32) | w[3];
    s_rnd[2 * plane + t] = ((u64)w[4] << 32) | w[5];
  }
  __syncthreads();
  // Update phase.  A thread keeps one (replica, slot) column (lg) for the
  // whole loop -- its three random words stay in registers per site -- and
  // walks (site of the tile, sample word) with a stride of nth/G groups, so
  // the G lanes of a group touch the G consecutive words of one site.
  const int G = NR * NB;
  const size_t wps = (size_t)V * G;  // words per sample word
  const int nk = min(kt, n - k0), nidx = nk * d.nw;
  if ((NB & 1) == 0) {
    // even NB: a lane takes two adjacent slots of a (replica, site) with
    // 16-byte loads and stores (every word offset here is even)
    const int G2 = G >> 1, NB2 = NB >> 1;
    const size_t wps2 = wps >> 1;
    for (int lg = tid % G2, grp = tid / G2, ngrp = max(1, nth / G2); lg < G2; lg += (nth >= G2 ? G2 : nth)) {
      if (nth >= G2 && grp >= ngrp) break;
      const int b = 2 * (lg % NB2), r = lg / NB2;
      ulonglong2 *Sc = reinterpret_cast<ulonglong2 *>(d.S + r * NB + b);
      const int step = nth >= G2 ? ngrp : 1;
      int idx = nth >= G2 ? grp : 0, kk = idx % nk, w = idx / nk;
      for (; idx < nidx; idx += step) {
        const int *sn = s_nb + kk * 7;
        const int site = sn[0];
        ulonglong2 *Sw = Sc + (size_t)w * wps2;
        const u64 *Jp = d.J + ((size_t)w * V + site) * 6;
        const ulonglong2 sv = Sw[(size_t)site * G2];
        u64 f0[6], f1[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          const u64 jq = __ldg(Jp + q);
          const ulonglong2 nq = Sw[(size_t)sn[q + 1] * G2];
          f0[q] = sv.x ^ jq ^ nq.x;
          f1[q] = sv.y ^ jq ^ nq.y;
        }
        const int o = (kk * NR + r) * NB + b;
        const ulonglong2 r0 = *reinterpret_cast<const ulonglong2 *>(s_rnd + o);
        const ulonglong2 r1 = *reinterpret_cast<const ulonglong2 *>(s_rnd + plane + o);
        const ulonglong2 r2 = *reinterpret_cast<const ulonglong2 *>(s_rnd + 2 * plane + o);
        ulonglong2 out;
        out.x = sv.x ^ flip_mask(f0, r0.x, r1.x, r2.x);
        out.y = sv.y ^ flip_mask(f1, r0.y, r1.y, r2.y);
        Sw[(size_t)site * G2] = out;
        for (kk += step; kk >= nk; kk -= nk) ++w;
      }
    }
    return;
  }
  for (int lg = tid % G, grp = tid / G, ngrp = max(1, nth / G); lg < G; lg += (nth >= G ? G : nth)) {
    if (nth >= G && grp >= ngrp) break;
    const int b = lg % NB, r = lg / NB;
    u64 *Sc = d.S + lg;
    const int step = nth >= G ? ngrp : 1;
    int idx = nth >= G ? grp : 0, kk = idx % nk, w = idx / nk;
    for (; idx < nidx; idx += step) {
      const int *sn = s_nb + kk * 7;
      const int site = sn[0];
      u64 *Sw = Sc + (size_t)w * wps;
      const u64 *Jp = d.J + ((size_t)w * V + site) * 6;
      const u64 sv = Sw[(size_t)site * G];
      u64 f[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) f[q] = sv ^ __ldg(Jp + q) ^ Sw[(size_t)sn[q + 1] * G];
      const int o = (kk * NR + r) * NB + b;
      Sw[(size_t)site * G] = sv ^ flip_mask(f, s_rnd[o], s_rnd[plane + o], s_rnd[2 * plane + o]);
      for (kk += step; kk >= nk; kk -= nk) ++w;
    }
  }
}

// The per-item form of a colour pass.  A thread takes (site, replica, slot)
// items of the colour in turn -- consecutive lanes on consecutive slots, so a
// warp's loads and stores cover consecutive words -- draws the item's three
// random words and updates the item's word in each sample word.  The block
// stages the 11-bit pre-search tables once (the thresholds, rarely read past
// them, come through the read-only cache); no random word goes through SMEM
// and no barrier separates drawing from updating.  The words are those of the
// tiles (same random words per (slot, site, replica), same flip mask).  This
// form suits jobs with few sample words, whose tiles spend their time on
// barriers and SMEM traffic for random words used once.
// The thread takes items t0, t0 + stride, ... below tend of the colour's
// n x NR x NB (the block's threads take consecutive t0): one job runs it on
// a grid of resident CTAs (k_sp_pass_items), a batch on 4 x 512 items a
// block (sp_pass_any).
__device__ __forceinline__ void sp_pass_items_body(const SpDev &d, int off, int n, long long t0, long long tend,
                                                   long long stride, unsigned char *smem) {
  const int NB = d.NB, NR = d.NR, G = NR * NB, V = d.V;
  uint8_t *s_pre = smem;
  {
    const uint4 *ps = reinterpret_cast<const uint4 *>(d.pre11);
    uint4 *pd = reinterpret_cast<uint4 *>(s_pre);
    for (int i = threadIdx.x; i < NB * (kPre11Stride / 16); i += blockDim.x) pd[i] = ps[i];
  }
  __syncthreads();
  const long long t1 = min(tend, (long long)n * G);
  const size_t wps = (size_t)V * G;  // words per sample word
  for (long long t = t0; t < t1; t += stride) {
    const int b = (int)(t % NB), r = (int)((t / NB) % NR), k = (int)(t / G);
    const int site = __ldg(d.col_sites + off + k);
    const uint32_t tp = (uint32_t)(((size_t)b * V + site) * NR + r);
    const uint4 c = d.ctr[r];
    const uint32_t key = __ldg(d.keys + r);
    const u64 *cum = d.cum + b * 256;
    const uint8_t *pre = s_pre + b * kPre11Stride;
    uint32_t w[6];
#pragma unroll
    for (int q = 0; q < 6; ++q)
      w[q] = rnd_word_by(c.x + q, c.y, c.z + tp, c.w, key, tp,
                         [&](uint32_t hi, uint32_t lo) { return lut_byte11(hi, lo, cum, pre); });
    const u64 r0 = ((u64)w[0] << 32) | w[1], r1 = ((u64)w[2] << 32) | w[3], r2 = ((u64)w[4] << 32) | w[5];
    int nbr[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) nbr[q] = __ldg(d.nb + (size_t)site * 6 + q);
    u64 *Sc = d.S + (size_t)r * NB + b;
    for (int ww = 0; ww < d.nw; ++ww) {
      u64 *Sw = Sc + (size_t)ww * wps;
      const u64 *Jp = d.J + ((size_t)ww * V + site) * 6;
      const u64 sv = Sw[(size_t)site * G];
      u64 f[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) f[q] = sv ^ __ldg(Jp + q) ^ Sw[(size_t)nbr[q] * G];
      Sw[(size_t)site * G] = sv ^ flip_mask(f, r0, r1, r2);
    }
  }
}

// A job's colour pass by its form; blk counts the job's blocks of the pass
// (tiles, or kItemsPerThread x blockDim.x items of the per-item form).
constexpr int kItemsPerThread = 4;
__device__ __forceinline__ void sp_pass_any(const SpDev &d, int colour, int blk, unsigned char *smem) {
  const int off = d.col_off[colour], n = d.col_off[colour + 1] - off;
  if (d.pgrid) {
    const long long t0 = (long long)blk * blockDim.x * kItemsPerThread;
    sp_pass_items_body(d, off, n, t0 + threadIdx.x, t0 + (long long)blockDim.x * kItemsPerThread, blockDim.x, smem);
  } else {
    sp_pass_body(d, off, n, blk, smem);
  }
}

// ---------------------------------------------------------------------------
// Energy: per (word, sample, replica, slot) the number of unsatisfied
// half-edges U2 (each bond counted from both ends), so E = 3V - U2
// (main.cu:1379).  A thread owns one (replica, slot) column of a word over a
// chunk of sites and counts the unsatisfied slots of each sample with
// bit-sliced counters (one bit plane per power of two, all 64 samples at
// once), then adds its per-sample totals to U2.
// ---------------------------------------------------------------------------
constexpr int kSpChunkMax = 256;  // sites per thread: 6 * 256 < 2^11
constexpr int kSpPlanes = 11;

// Sites per thread of the energy kernel: enough threads to fill the GPU
// (152 SMs x 2048), at least 4 sites each (each thread ends with up to 64
// atomic additions, which small chunks pile on the same counters).  Jobs too
// small to fill the GPU get the floor: their count is a chain of dependent
// loads per site, so fewer sites a thread is a shorter chain (16 sites a
// thread measured 16-21 us per count on one-word jobs).
int sp_energy_chunk(const SpDev &d) {
  const double words = (double)d.nw * d.esites * d.NR * d.NB;
  int c = (int)(words / (152.0 * 2048.0));
  return c < 4 ? 4 : (c > kSpChunkMax ? kSpChunkMax : c);
}

// col: the thread's index over nw * nchunk * G (blocks of 256 threads).
// With epair (two colours, both ends of every bond holding its coupling word:
// checked on the host when the couplings are set) every bond has exactly one
// colour-1 end, so the count walks the colour-1 sites only and doubles them.
__device__ __forceinline__ void sp_energy_body(const SpDev &d, long long col) {
  const int G = d.NR * d.NB, V = d.V, chunk = d.echunk, ns = d.esites;
  const int nchunk = (ns + chunk - 1) / chunk;
  if (col >= (long long)d.nw * nchunk * G) return;
  const int rb = (int)(col % G), ch = (int)((col / G) % nchunk), w = (int)(col / ((long long)G * nchunk));
  const u64 *Sw = d.S + (size_t)w * V * G + rb;
  const u64 *Jw = d.J + (size_t)w * V * 6;
  u64 P[kSpPlanes];
#pragma unroll
  for (int p = 0; p < kSpPlanes; ++p) P[p] = 0;
  const int i0 = ch * chunk, i1 = min(ns, i0 + chunk);
  const int32_t *c1 = d.col_sites + d.col_off[1];
  // two sites an iteration, so that the second site's loads are in flight
  // while the first is counted (the words are read-only here)
#pragma unroll 2
  for (int ii = i0; ii < i1; ++ii) {
    const int i = d.epair ? __ldg(c1 + ii) : ii;
    const u64 sv = __ldg(Sw + (size_t)i * G);
    const int *nb = d.nb + (size_t)i * 6;
    u64 f[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) f[q] = sv ^ __ldg(Jw + (size_t)i * 6 + q) ^ __ldg(Sw + (size_t)__ldg(nb + q) * G);
    // six bits -> a 3-bit count per sample (two full adders and a merge)
    const u64 x1 = f[0] ^ f[1] ^ f[2], y1 = (f[0] & f[1]) | (f[2] & (f[0] ^ f[1]));
    const u64 x2 = f[3] ^ f[4] ^ f[5], y2 = (f[3] & f[4]) | (f[5] & (f[3] ^ f[4]));
    const u64 z0 = x1 ^ x2, c0 = x1 & x2;
    const u64 z1 = y1 ^ y2 ^ c0, z2 = (y1 & y2) | (c0 & (y1 ^ y2));
    // add z0 + 2 z1 + 4 z2 to the counter planes
    u64 c = P[0] & z0;
    P[0] ^= z0;
    u64 s = P[1] ^ z1 ^ c;
    c = (P[1] & z1) | (c & (P[1] ^ z1));
    P[1] = s;
    s = P[2] ^ z2 ^ c;
    c = (P[2] & z2) | (c & (P[2] ^ z2));
    P[2] = s;
#pragma unroll
    for (int p = 3; p < kSpPlanes; ++p) {
      const u64 t = P[p] & c;
      P[p] ^= c;
      c = t;
    }
  }
  int32_t *U = d.U2 + (size_t)w * 64 * G + rb;
  int np = kSpPlanes;
  while (np > 1 && !P[np - 1]) --np;
  for (int lane = 0; lane < 64; ++lane) {
    int cnt = 0;
    for (int p = 0; p < np; ++p) cnt |= (int)((P[p] >> lane) & 1ull) << p;
    if (cnt) atomicAdd(U + (size_t)lane * G, cnt << d.epair);
  }
}

// ---------------------------------------------------------------------------
// Tempering: one thread per (word, sample, replica) chain; the rule of
// upd.c:3-48 over the slot pairs in order (pt = -(b[i+1]-b[i]) * dE in FP64,
// accept when pt >= 0 or FNORM * u < exp(pt), exp from the host's libm table;
// beyond the table exp(pt) < 2^-72 and only u = 0 accepts).  The 64-bit
// uniform u of (step, pair, chain) is Philox4x32-10 keyed by the job's
// tempering seed -- the reference draws it from a per-chain Parisi-Rapuano
// generator; sample-packed jobs have 64 chains per word, so a counter-based
// draw replaces the 2 KB of state per chain.  A warp holds 32 samples of one
// (word, replica): the accepted swaps of pair i form the lane mask M[i].
// ---------------------------------------------------------------------------
// wr = (word, replica); lane = sample, 0..63, the 64 lanes two whole warps.
__device__ __forceinline__ void sp_pt_body(const SpDev &d, int wr, int lane) {
  const int NB = d.NB, NR = d.NR, G = NR * NB;
  const int w = wr / NR, r = wr % NR;
  const int nt = 3 * d.V;
  const size_t o = ((size_t)w * 64 + lane) * G + (size_t)r * NB;
  const unsigned long long step = *d.ptstep;
  const uint32_t chain = (uint32_t)(((size_t)w * 64 + lane) * NR + r);
  const double FNORM = 5.4210108624275218e-20;
  uint32_t *acc = d.acc + ((size_t)w * 64 + lane) * NR * (NB - 1) + (size_t)r * (NB - 1);
  uint32_t *Mh = reinterpret_cast<uint32_t *>(d.M + ((size_t)w * NR + r) * (NB - 1));
  // The pairs in order: slot i+1 still holds its own configuration when pair
  // i is decided, slot i holds the one carried up from below (a swap at i
  // moves it on to i+1).  So the chain keeps only the carried energy and id
  // in registers; slot i's final values are written as soon as pair i is
  // decided.
  int carry_e = nt - d.U2[o];
  uint8_t carry_p = d.perm[o];
  for (int i = 0; i < NB - 1; ++i) {
    const int e1 = nt - d.U2[o + i + 1];
    const uint8_t p1 = d.perm[o + i + 1];
    const int dE = e1 - carry_e;
    const double pt = __dmul_rn(-__dsub_rn(d.betas[i + 1], d.betas[i]), (double)dE);
    uint32_t v0 = (uint32_t)step, v1 = (uint32_t)(step >> 32), v2 = (uint32_t)i, v3 = chain;
    philox10(v0, v1, v2, v3, (uint32_t)d.pt_seed, (uint32_t)(d.pt_seed >> 32));
    const u64 u = ((u64)v0 << 32) | v1;
    bool change;
    if (pt >= 0.0) {
      change = true;
    } else {
      const int base = d.expoff[i], m = (-dE) >> 1, nx = d.expoff[i + 1] - base;
      change = (m >= 1 && m <= nx) ? __dmul_rn(FNORM, __ull2double_rn(u)) < d.exptab[base + m - 1] : u == 0;
    }
    if (change) {
      d.E[o + i] = e1;
      d.perm[o + i] = p1;
      acc[i] += 1u;
    } else {
      d.E[o + i] = carry_e;
      d.perm[o + i] = carry_p;
      carry_e = e1;
      carry_p = p1;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, change);
    if ((lane & 31) == 0) Mh[2 * i + (lane >> 5)] = mask;
  }
  d.E[o + NB - 1] = carry_e;
  d.perm[o + NB - 1] = carry_p;
}

// The accepted swaps of the last tempering step, applied to the words in
// pair order: slot i exchanges the masked samples with slot i+1, and is final
// after that (one carry word).  A block stages kPermRows consecutive
// (word, site, replica) rows of NB words through SMEM, so that global loads
// and stores are coalesced, and each thread then walks one row.
constexpr int kPermRows = 128;

__device__ __forceinline__ void sp_permute_body(const SpDev &d, int blk, u64 *rows) {
  const int NB = d.NB, NR = d.NR;
  const long long nrows = (long long)d.nw * d.V * NR;
  const long long r0 = (long long)blk * kPermRows;
  if (blk == 0 && threadIdx.x == 0) *d.ptstep += 1ull;
  const int nr = (int)min((long long)kPermRows, nrows - r0);
  // rows sit in SMEM with an odd stride (in words): the threads' scans then
  // hit distinct banks (an even stride such as NB = 24 is a 16-way conflict)
  const int rs = NB | 1;
  u64 *g = d.S + (size_t)r0 * NB;
  for (int k = threadIdx.x; k < nr * NB; k += blockDim.x) {
    const int row = k / NB;
    rows[row * rs + (k - row * NB)] = g[k];
  }
  __syncthreads();
  if (threadIdx.x < nr) {
    const long long t = r0 + threadIdx.x;
    const int r = (int)(t % NR), w = (int)(t / ((long long)NR * d.V));
    u64 *p = rows + (size_t)threadIdx.x * rs;
    const u64 *M = d.M + ((size_t)w * NR + r) * (NB - 1);
    u64 cur = p[0];
    for (int i = 0; i < NB - 1; ++i) {
      const u64 m = __ldg(M + i);
      const u64 nxt = p[i + 1];
      const u64 x = (cur ^ nxt) & m;
      p[i] = cur ^ x;
      cur = nxt ^ x;
    }
    p[NB - 1] = cur;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nr * NB; k += blockDim.x) {
    const int row = k / NB;
    g[k] = rows[row * rs + (k - row * NB)];
  }
}


// ---------------------------------------------------------------------------
// Houdayer move (main.cu:351-453, HoudayerXEA.cu:54-374), per sample.
// Replica pairs: as the reference picks them (main.cu:408-421) from random_c,
// in two groups of NR/2 replicas (one group of NR when NR < 4).  For each
// group and each slot b < nclust, the overlap q = s_r1 ^ s_r2 of every sample
// is split into maximal clusters of equal q along all six bond slots (the
// fake bonds of open planes included, so every move conserves E(r1)+E(r2)
// for any L; for even L the fake bonds duplicate y bonds and the clusters
// are the reference's); a cluster's root is its smallest site index, as in
// the reference, and each cluster flips in both replicas with probability
// 1/2.  The coin of a cluster is the lowest bit of Philox4x32-10 of (move,
// root, sample, slot, group) -- the reference compares a cuRAND uniform per
// (sample, beta, root) with 0.5 (HoudayerXEA.cu:373); a counter-based bit
// needs no V*NB uniforms per sample.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sp_pairs_body(const SpDev &d) {
  *d.move += 1ull;
  const int ng = d.NR >= 4 ? 2 : 1, h = d.NR / ng;
  for (int g = 0; g < ng; ++g) {
    int idx[64];
    for (int k = 0; k < h; ++k) idx[k] = k + g * h;
    for (int k = 0; k < h - 1; ++k) {
      const u64 f = d_hq_next(d.rc);
      const int q = k + (int)(((uint32_t)(f >> 32)) % (uint32_t)(h - k));
      const int t = idx[k]; idx[k] = idx[q]; idx[q] = t;
    }
    d.pairs[2 * g] = idx[0];
    d.pairs[2 * g + 1] = idx[1];
  }
}

__device__ __forceinline__ void sp_overlap_body(const SpDev &d, int g, long long t) {  // t = (w, b, site)
  const int V = d.V, nc = d.nclust;
  if (t >= (long long)d.nw * nc * V) return;
  const int i = (int)(t % V), b = (int)((t / V) % nc), w = (int)(t / ((long long)V * nc));
  const int r1 = d.pairs[2 * g], r2 = d.pairs[2 * g + 1];
  const u64 *p = d.S + (((size_t)w * V + i) * d.NR) * d.NB + b;
  d.Q[t] = p[(size_t)r1 * d.NB] ^ p[(size_t)r2 * d.NB];
}

// One CTA per (word, slot, group of 8 samples): the CTA reads its byte of
// every site's overlap word into SMEM and labels the 8 samples' lattices one
// after the other with lock-step rounds -- each site hooks the labels of its
// equal-q neighbours of smaller index with atomicMin, then labels are
// pointer-jumped until stable, until a round hooks nothing.  Labels only
// decrease and stay inside the cluster, so each cluster ends labelled by its
// smallest site.  The roots' coins give the samples' flip bits, gathered per
// site in a byte that replaces the CTA's byte of the overlap word (the 8
// groups of a word own disjoint bytes, so no atomics); k_sp_flip then applies
// the flip words to both replicas.
// Lattices above kSpClusterMaxV sites keep the same arrays in a global
// scratch region of the CTA (L2-resident) instead of SMEM.
// Key of the cluster coins of a job: its tempering seed, offset.
__host__ __device__ inline unsigned long long sp_cluster_key(const SpDev &d) { return d.pt_seed ^ 0xC2B2AE3585EBCA6BULL; }

__device__ __forceinline__ void sp_cluster_body(const SpDev &d, int g, int blk, uint32_t *sm) {
  const unsigned long long key = sp_cluster_key(d);
  const int V = d.V, nc = d.nclust;
  uint32_t *base = V <= kSpClusterMaxV ? sm : d.cscratch + (size_t)blk * sp_cluster_words(V);
  uint32_t *lab = base;                                              // [V]
  uint8_t *qb = reinterpret_cast<uint8_t *>(lab + V);                // [V] q bits of the 8 samples
  uint8_t *fb = qb + V;                                              // [V] flip bits of the 8 samples
  uint8_t *bond = fb + V;                                            // [V] equal-q slots to smaller sites
  const int grp = blk & 7, lat = blk >> 3;                           // lat = w * nc + b
  const int b = lat % nc, w = lat / nc;
  uint8_t *Qb = reinterpret_cast<uint8_t *>(d.Q + (size_t)lat * V) + grp;
  for (int i = threadIdx.x; i < V; i += blockDim.x) {
    qb[i] = Qb[(size_t)i * 8];
    fb[i] = 0;
  }
  __syncthreads();
  const unsigned long long mv = *d.move;
  for (int l = 0; l < 8; ++l) {
    for (int i = threadIdx.x; i < V; i += blockDim.x) {
      const unsigned qi = (qb[i] >> l) & 1u;
      unsigned m = 0;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const int p = __ldg(d.nb + (size_t)i * 6 + q);
        if (p < i && ((qb[p] >> l) & 1u) == qi) m |= 1u << q;
      }
      bond[i] = (uint8_t)m;
      lab[i] = (uint32_t)i;
    }
    __syncthreads();
    for (;;) {
      int hooked = 0;
      for (int i = threadIdx.x; i < V; i += blockDim.x) {
        const unsigned m = bond[i];
        if (!m) continue;
        const uint32_t li = lab[i];
#pragma unroll
        for (int q = 0; q < 6; ++q)
          if ((m >> q) & 1u) {
            const uint32_t lj = lab[__ldg(d.nb + (size_t)i * 6 + q)];
            if (lj != li) { atomicMin(&lab[max(li, lj)], min(li, lj)); hooked = 1; }
          }
      }
      if (!__syncthreads_or(hooked)) break;
      for (;;) {
        int moved = 0;
        for (int i = threadIdx.x; i < V; i += blockDim.x) {
          const uint32_t x = lab[i], y = lab[x];
          if (y != x) { lab[i] = y; moved = 1; }
        }
        if (!__syncthreads_or(moved)) break;
      }
    }
    // coins of the roots, kept in the roots' bond bytes (no longer needed)
    const int lane = grp * 8 + l;
    const uint32_t tag = (((uint32_t)(w * 64 + lane) << 6 | (uint32_t)b) << 1) | (uint32_t)g;
    for (int i = threadIdx.x; i < V; i += blockDim.x) {
      if (lab[i] != (uint32_t)i) continue;
      uint32_t v0 = (uint32_t)mv, v1 = (uint32_t)(mv >> 32), v2 = (uint32_t)i, v3 = tag;
      philox10(v0, v1, v2, v3, (uint32_t)key, (uint32_t)(key >> 32));
      bond[i] = (uint8_t)(v0 & 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < V; i += blockDim.x) fb[i] |= (uint8_t)(bond[lab[i]] << l);
    __syncthreads();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < V; i += blockDim.x) Qb[(size_t)i * 8] = fb[i];
}

// The same labelling for 4 samples at a time, for lattices up to
// kSpCluster4MaxV sites: a site's 4 labels sit in one 16-byte SMEM slot and
// its 4 bond masks in one word (sample l at bits 8l..8l+5), so that one
// neighbour-table load and one loop step serve the 4 samples (the 1-sample
// form spends ~600 instructions per site and lattice, mostly on those).
// Roots, coins and flip bytes are those of sp_cluster_body.
__device__ __forceinline__ uint32_t spread4(uint32_t x) {
  return (x & 1u) | ((x & 2u) << 7) | ((x & 4u) << 14) | ((x & 8u) << 21);
}

__device__ __forceinline__ void sp_cluster4_body(const SpDev &d, int g, int blk, uint32_t *sm) {
  const unsigned long long key = sp_cluster_key(d);
  const int V = d.V, nc = d.nclust;
  uint4 *lab = reinterpret_cast<uint4 *>(sm);                          // [V]
  uint32_t *lab1 = sm;                                                 // the same, one label per word
  uint32_t *bond = sm + 4 * (size_t)V;                                 // [V]
  uint8_t *qb = reinterpret_cast<uint8_t *>(bond + V);                 // [V]
  uint8_t *fb = qb + V;                                                // [V]
  const int grp = blk & 7, lat = blk >> 3;
  const int b = lat % nc, w = lat / nc;
  uint8_t *Qb = reinterpret_cast<uint8_t *>(d.Q + (size_t)lat * V) + grp;
  for (int i = threadIdx.x; i < V; i += blockDim.x) {
    qb[i] = Qb[(size_t)i * 8];
    fb[i] = 0;
  }
  __syncthreads();
  const unsigned long long mv = *d.move;
  for (int h = 0; h < 2; ++h) {
    for (int i = threadIdx.x; i < V; i += blockDim.x) {
      const uint32_t qi = (qb[i] >> (4 * h)) & 15u;
      uint32_t m = 0;
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const int p = __ldg(d.nb + (size_t)i * 6 + q);
        if (p < i) m |= spread4(~(qi ^ (qb[p] >> (4 * h))) & 15u) << q;
      }
      bond[i] = m;
      lab[i] = make_uint4((uint32_t)i, (uint32_t)i, (uint32_t)i, (uint32_t)i);
    }
    __syncthreads();
    for (;;) {
      int hooked = 0;
      for (int i = threadIdx.x; i < V; i += blockDim.x) {
        const uint32_t m = bond[i];
        if (!m) continue;
        const uint4 li4 = lab[i];
        const uint32_t li[4] = {li4.x, li4.y, li4.z, li4.w};
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          const uint32_t mq = (m >> q) & 0x01010101u;
          if (!mq) continue;
          const int p = __ldg(d.nb + (size_t)i * 6 + q);
          const uint4 lj4 = lab[p];
          const uint32_t lj[4] = {lj4.x, lj4.y, lj4.z, lj4.w};
#pragma unroll
          for (int l = 0; l < 4; ++l)
            if (((mq >> (8 * l)) & 1u) && lj[l] != li[l]) {
              atomicMin(&lab1[4 * (size_t)max(li[l], lj[l]) + l], min(li[l], lj[l]));
              hooked = 1;
            }
        }
      }
      if (!__syncthreads_or(hooked)) break;
      for (;;) {
        int moved = 0;
        for (int i = threadIdx.x; i < V; i += blockDim.x) {
          const uint4 x = lab[i];
          const uint4 y = make_uint4(lab1[4 * (size_t)x.x], lab1[4 * (size_t)x.y + 1], lab1[4 * (size_t)x.z + 2],
                                     lab1[4 * (size_t)x.w + 3]);
          if (y.x != x.x || y.y != x.y || y.z != x.z || y.w != x.w) { lab[i] = y; moved = 1; }
        }
        if (!__syncthreads_or(moved)) break;
      }
    }
    // coins of the roots (bits 0..3 of the roots' bond words, no longer needed)
    for (int i = threadIdx.x; i < V; i += blockDim.x) {
      const uint4 x = lab[i];
      const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
      uint32_t c = 0;
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        if (xs[l] != (uint32_t)i) continue;
        const int lane = grp * 8 + 4 * h + l;
        const uint32_t tag = (((uint32_t)(w * 64 + lane) << 6 | (uint32_t)b) << 1) | (uint32_t)g;
        uint32_t v0 = (uint32_t)mv, v1 = (uint32_t)(mv >> 32), v2 = (uint32_t)i, v3 = tag;
        philox10(v0, v1, v2, v3, (uint32_t)key, (uint32_t)(key >> 32));
        c |= (v0 & 1u) << l;
      }
      bond[i] = c;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < V; i += blockDim.x) {
      const uint4 x = lab[i];
      const uint32_t f = (bond[x.x] & 1u) | (bond[x.y] & 2u) | (bond[x.z] & 4u) | (bond[x.w] & 8u);
      fb[i] |= (uint8_t)(f << (4 * h));
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < V; i += blockDim.x) Qb[(size_t)i * 8] = fb[i];
}

// The same labelling for all 8 samples of the CTA at once, for lattices up
// to kSpCluster8MaxV sites: 16-bit labels, a site's 8 in one 16-byte SMEM
// slot, its 8 bond masks in one 64-bit word (sample l at bits 8l..8l+5), so
// one neighbour-table load and one loop step serve the 8 samples, in a single
// pass (26 bytes of SMEM per site).  SMEM has no 16-bit atomicMin, so a hook
// is a plain store: when several threads hook one root in a round, one
// store stays and the other bonds are hooked again in the next round, as
// with atomicMin (which keeps one link per root and round as well).  Every
// value stored is a smaller site of the same cluster, so labels still end at
// each cluster's smallest site.
constexpr int kSpCluster8MaxV = 8900;

__device__ __forceinline__ unsigned long long spread8(uint32_t x) {
  unsigned long long r = 0;
#pragma unroll
  for (int l = 0; l < 8; ++l) r |= (unsigned long long)((x >> l) & 1u) << (8 * l);
  return r;
}

__device__ __forceinline__ void unpack8(uint4 v, uint32_t l[8]) {
  l[0] = v.x & 0xFFFFu; l[1] = v.x >> 16; l[2] = v.y & 0xFFFFu; l[3] = v.y >> 16;
  l[4] = v.z & 0xFFFFu; l[5] = v.z >> 16; l[6] = v.w & 0xFFFFu; l[7] = v.w >> 16;
}

__device__ __forceinline__ uint4 pack8(const uint32_t l[8]) {
  return make_uint4(l[0] | (l[1] << 16), l[2] | (l[3] << 16), l[4] | (l[5] << 16), l[6] | (l[7] << 16));
}

// The 8-sample lock-step labelling of the sites [base, base + Vs) (all of
// the lattice, or one slab of z planes): bonds to sites outside the run are
// left out; labels are local indices (site - base).  SMEM: lab [Vs] (8
// labels a site), bond [Vs], qb [Vs] (the group's 8 q bits a site).
__device__ __forceinline__ void sp_label8(const SpDev &d, const uint8_t *Qb, int base, int Vs, unsigned char *sm) {
  uint4 *lab = reinterpret_cast<uint4 *>(sm);
  uint16_t *lab16 = reinterpret_cast<uint16_t *>(sm);
  unsigned long long *bond = reinterpret_cast<unsigned long long *>(sm + (size_t)16 * Vs);
  uint8_t *qb = sm + (size_t)24 * Vs;
  for (int i = threadIdx.x; i < Vs; i += blockDim.x) qb[i] = Qb[(size_t)(base + i) * 8];
  __syncthreads();
  for (int i = threadIdx.x; i < Vs; i += blockDim.x) {
    const uint32_t qi = qb[i];
    const int gi = base + i;
    unsigned long long m = 0;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const int p = __ldg(d.nb + (size_t)gi * 6 + q);
      if (p >= base && p < gi) m |= spread8(~(qi ^ qb[p - base]) & 0xFFu) << q;
    }
    bond[i] = m;
    const uint32_t ii = (uint32_t)i | ((uint32_t)i << 16);
    lab[i] = make_uint4(ii, ii, ii, ii);
  }
  __syncthreads();
  const int V = Vs;
  for (;;) {
    int hooked = 0;
    for (int i = threadIdx.x; i < V; i += blockDim.x) {
      const unsigned long long m = bond[i];
      if (!m) continue;
      uint32_t li[8];
      unpack8(lab[i], li);
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const unsigned long long mq = (m >> q) & 0x0101010101010101ull;
        if (!mq) continue;
        const int p = __ldg(d.nb + (size_t)(base + i) * 6 + q) - base;
        uint32_t lj[8];
        unpack8(lab[p], lj);
#pragma unroll
        for (int l = 0; l < 8; ++l)
          if (((mq >> (8 * l)) & 1ull) && lj[l] != li[l]) {
            lab16[8 * (size_t)max(li[l], lj[l]) + l] = (uint16_t)min(li[l], lj[l]);
            hooked = 1;
          }
      }
    }
    if (!__syncthreads_or(hooked)) break;
    for (;;) {
      int moved = 0;
      for (int i = threadIdx.x; i < V; i += blockDim.x) {
        uint32_t x[8], y[8];
        unpack8(lab[i], x);
        bool ch = false;
#pragma unroll
        for (int l = 0; l < 8; ++l) {
          y[l] = lab16[8 * (size_t)x[l] + l];
          ch |= y[l] != x[l];
        }
        if (ch) { lab[i] = pack8(y); moved = 1; }
      }
      if (!__syncthreads_or(moved)) break;
    }
  }
}

__device__ __forceinline__ void sp_cluster8_body(const SpDev &d, int g, int blk, unsigned char *sm) {
  const unsigned long long key = sp_cluster_key(d);
  const int V = d.V, nc = d.nclust;
  uint4 *lab = reinterpret_cast<uint4 *>(sm);                                  // [V]: 8 labels
  uint8_t *qb = sm + (size_t)24 * V;                                           // [V] q bits, then coins
  const int grp = blk & 7, lat = blk >> 3;
  const int b = lat % nc, w = lat / nc;
  uint8_t *Qb = reinterpret_cast<uint8_t *>(d.Q + (size_t)lat * V) + grp;
  sp_label8(d, Qb, 0, V, sm);
  // coins of the roots (in qb, no longer needed), then the flip bytes
  const unsigned long long mv = *d.move;
  for (int i = threadIdx.x; i < V; i += blockDim.x) {
    uint32_t x[8];
    unpack8(lab[i], x);
    uint32_t c = 0;
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      if (x[l] != (uint32_t)i) continue;
      const int lane = grp * 8 + l;
      const uint32_t tag = (((uint32_t)(w * 64 + lane) << 6 | (uint32_t)b) << 1) | (uint32_t)g;
      uint32_t v0 = (uint32_t)mv, v1 = (uint32_t)(mv >> 32), v2 = (uint32_t)i, v3 = tag;
      philox10(v0, v1, v2, v3, (uint32_t)key, (uint32_t)(key >> 32));
      c |= (v0 & 1u) << l;
    }
    qb[i] = (uint8_t)c;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < V; i += blockDim.x) {
    uint32_t x[8];
    unpack8(lab[i], x);
    uint32_t f = 0;
#pragma unroll
    for (int l = 0; l < 8; ++l) f |= ((uint32_t)(qb[x[l]] >> l) & 1u) << l;
    Qb[(size_t)i * 8] = (uint8_t)f;
  }
}

// ---------------------------------------------------------------------------
// Lattices above kSpClusterMaxV sites, one-job path: slabs of slabD z planes
// labelled 8 samples at a time in SMEM (sp_label8), each site's label written
// as a global site index into slab_lab [unit = lattice * 8 + group][8][V];
// then the bonds between slabs joined by the lock-free union of the
// multispin path (cc_unite: a root hung below the smaller one with
// atomicMin), the labels compressed to their roots and the roots' coins
// drawn (slab_coin [unit][V], one bit a sample), and the flip bytes written
// in place of the overlap bytes.  Labels only decrease and never drop below
// the smallest site of their cluster, so the roots -- and the coins and
// flips -- are those of the one-CTA labelling.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sp_slab8_body(const SpDev &d, int unit, int sl, unsigned char *sm) {
  const int V = d.V, L2 = d.L * d.L, z0 = sl * d.slabD;
  const int base = z0 * L2, Vs = min(d.slabD, d.Lz - z0) * L2;
  const int grp = unit & 7, lat = unit >> 3;
  const uint8_t *Qb = reinterpret_cast<const uint8_t *>(d.Q + (size_t)lat * V) + grp;
  sp_label8(d, Qb, base, Vs, sm);
  const uint4 *lab = reinterpret_cast<const uint4 *>(sm);
  uint32_t *Lu = d.slab_lab + (size_t)unit * 8 * V;
  for (int i = threadIdx.x; i < Vs; i += blockDim.x) {
    uint32_t x[8];
    unpack8(lab[i], x);
#pragma unroll
    for (int l = 0; l < 8; ++l) Lu[(size_t)l * V + base + i] = (uint32_t)(base + (int)x[l]);
  }
}

// Bonds between slabs (each once, from its larger end): t = unit * V + site.
__device__ __forceinline__ void sp_slab_merge_body(const SpDev &d, long long t) {
  const int V = d.V, L2 = d.L * d.L;
  if (t >= (long long)d.nw * d.nclust * 8 * V) return;
  const int unit = (int)(t / V), gi = (int)(t - (long long)unit * V);
  const int grp = unit & 7, lat = unit >> 3;
  const uint8_t *Qb = reinterpret_cast<const uint8_t *>(d.Q + (size_t)lat * V) + grp;
  const int s1 = gi / L2 / d.slabD;
  const uint32_t qi = Qb[(size_t)gi * 8];
  uint32_t *Lu = d.slab_lab + (size_t)unit * 8 * V;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    const int p = __ldg(d.nb + (size_t)gi * 6 + q);
    if (p >= gi || p / L2 / d.slabD == s1) continue;
    const uint32_t eq = ~(qi ^ Qb[(size_t)p * 8]) & 0xFFu;
    for (int l = 0; l < 8; ++l)
      if ((eq >> l) & 1u) cc_unite(Lu + (size_t)l * V, (uint32_t)gi, (uint32_t)p);
  }
}

// Roots and their coins: t = unit * V + site.
__device__ __forceinline__ void sp_slab_roots_body(const SpDev &d, int g, long long t) {
  const int V = d.V, nc = d.nclust;
  if (t >= (long long)d.nw * nc * 8 * V) return;
  const int unit = (int)(t / V), gi = (int)(t - (long long)unit * V);
  const int grp = unit & 7, lat = unit >> 3, b = lat % nc, w = lat / nc;
  const unsigned long long key = sp_cluster_key(d), mv = *d.move;
  uint32_t *Lu = d.slab_lab + (size_t)unit * 8 * V;
  uint32_t coins = 0;
  for (int l = 0; l < 8; ++l) {
    const uint32_t r = cc_find(Lu + (size_t)l * V, (uint32_t)gi);
    Lu[(size_t)l * V + gi] = r;
    if (r != (uint32_t)gi) continue;
    const int lane = grp * 8 + l;
    const uint32_t tag = (((uint32_t)(w * 64 + lane) << 6 | (uint32_t)b) << 1) | (uint32_t)g;
    uint32_t v0 = (uint32_t)mv, v1 = (uint32_t)(mv >> 32), v2 = (uint32_t)gi, v3 = tag;
    philox10(v0, v1, v2, v3, (uint32_t)key, (uint32_t)(key >> 32));
    coins |= (v0 & 1u) << l;
  }
  d.slab_coin[(size_t)unit * V + gi] = (uint8_t)coins;
}

// Flip bytes from the roots' coins, in place of the overlap bytes.
__device__ __forceinline__ void sp_slab_flip_body(const SpDev &d, long long t) {
  const int V = d.V;
  if (t >= (long long)d.nw * d.nclust * 8 * V) return;
  const int unit = (int)(t / V), gi = (int)(t - (long long)unit * V);
  const int grp = unit & 7, lat = unit >> 3;
  const uint32_t *Lu = d.slab_lab + (size_t)unit * 8 * V;
  const uint8_t *Cu = d.slab_coin + (size_t)unit * V;
  uint32_t f = 0;
  for (int l = 0; l < 8; ++l) f |= (uint32_t)((Cu[Lu[(size_t)l * V + gi]] >> l) & 1u) << l;
  reinterpret_cast<uint8_t *>(d.Q + (size_t)lat * V)[(size_t)gi * 8 + grp] = (uint8_t)f;
}

// Labelling of one CTA's (word, slot, 8 samples) by lattice size.
__device__ __forceinline__ void sp_cluster_any(const SpDev &d, int g, int blk, unsigned char *sm) {
  if (d.V <= kSpCluster8MaxV) sp_cluster8_body(d, g, blk, sm);
  else if (d.V <= kSpCluster4MaxV) sp_cluster4_body(d, g, blk, reinterpret_cast<uint32_t *>(sm));
  else sp_cluster_body(d, g, blk, reinterpret_cast<uint32_t *>(sm));
}

// Both replicas of the group take the flip words: thread per (word, site, slot).
__device__ __forceinline__ void sp_flip_body(const SpDev &d, int g, long long t) {
  const int V = d.V, nc = d.nclust;
  if (t >= (long long)d.nw * V * nc) return;
  const int b = (int)(t % nc), i = (int)((t / nc) % V), w = (int)(t / ((long long)nc * V));
  const u64 F = d.Q[((size_t)w * nc + b) * V + i];
  if (!F) return;
  const int r1 = d.pairs[2 * g], r2 = d.pairs[2 * g + 1];
  u64 *p = d.S + (((size_t)w * V + i) * d.NR) * d.NB + b;
  p[(size_t)r1 * d.NB] ^= F;
  p[(size_t)r2 * d.NB] ^= F;
}

// Energy measurement of a bin's iteration: avgE += 3V - U2 (slot order).
// from_e: the measurement follows a tempering step directly (no cluster
// move in between), whose E already holds the energy of the configuration
// now at each slot (energies move with their configurations): no recount.
__device__ __forceinline__ void sp_measure_u2_body(const SpDev &d, long long i, int from_e) {
  if (i < (long long)d.nw * 64 * d.NR * d.NB) d.avgE[i] += from_e ? (double)d.E[i] : (double)(3 * d.V - d.U2[i]);
}

// ---------------------------------------------------------------------------
// Exact enumeration: for every sample of every word, the number of spin
// configurations at each energy E = 3V - U2 among the 2^(V-1) with spin 0 up
// (E is even under the global flip, so the full counts are twice these; the
// averages do not change).  Block row y = sample.  A thread walks 2^12
// configurations in Gray-code order from a prefix of the higher spins:
// flipping spin k changes U2 by 2 (6 - 2 n_k), n_k = unsatisfied slots at k.
// Counts go to a per-block SMEM histogram, then to the 64-bit global one.
// ---------------------------------------------------------------------------
constexpr int kDosLow = 12;

__global__ void __launch_bounds__(256) k_sp_dos(const __grid_constant__ SpDev d, int nprefix_bits) {
  __shared__ uint32_t h[6 * 32 + 1];
  const int V = d.V, nbins = 6 * V + 1;
  const int sample = blockIdx.y, w = sample / 64, lane = sample % 64;
  __shared__ int s_nb[32 * 6];
  __shared__ uint8_t s_j[32 * 6];
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) h[i] = 0;
  for (int i = threadIdx.x; i < V * 6; i += blockDim.x) {
    s_nb[i] = d.nb[i];
    s_j[i] = (uint8_t)((d.J[(size_t)w * V * 6 + i] >> lane) & 1ull);
  }
  __syncthreads();
  const int nlow = min(kDosLow, V - 1);
  const uint64_t prefix = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (prefix < (1ull << nprefix_bits)) {
    // configuration bits: spin 0 up (bit 0 = 0), spins 1..nlow by Gray code,
    // the rest from the prefix
    uint32_t s = (uint32_t)(prefix << (nlow + 1));
    auto unsat = [&](int k) {
      int n = 0;
      const int sk = (s >> k) & 1;
#pragma unroll
      for (int q = 0; q < 6; ++q) n += sk ^ (int)((s >> s_nb[k * 6 + q]) & 1u) ^ s_j[k * 6 + q];
      return n;
    };
    int U2 = 0;
    for (int k = 0; k < V; ++k) U2 += unsat(k);
    atomicAdd(&h[3 * V - U2 + 3 * V], 1u);
    for (uint32_t g = 1; g < (1u << nlow); ++g) {
      const int k = __ffs(g);  // Gray step g flips spin 1 + (trailing zeros of g)
      const int nk = unsat(k);
      U2 += 2 * (6 - 2 * nk);
      s ^= 1u << k;
      atomicAdd(&h[3 * V - U2 + 3 * V], 1u);
    }
  }
  __syncthreads();
  unsigned long long *out = d.dos + (size_t)sample * nbins;
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (h[i]) atomicAdd(out + i, (unsigned long long)h[i]);
}

// <E>(beta) of each sample from its density of states, in FP64: weights
// g(E) exp(beta (E - Emax)) over the bins.
__global__ void k_sp_exact(const __grid_constant__ SpDev d, const double *betas, int nbeta, double *meanE) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int V = d.V, nbins = 6 * V + 1;
  if (t >= d.nw * 64 * nbeta) return;
  const int sample = t / nbeta, k = t % nbeta;
  const unsigned long long *g = d.dos + (size_t)sample * nbins;
  int emax = -3 * V;
  for (int i = 0; i < nbins; ++i)
    if (g[i]) emax = i - 3 * V;
  double Z = 0, ZE = 0;
  for (int i = 0; i < nbins; ++i) {
    if (!g[i]) continue;
    const int E = i - 3 * V;
    const double wgt = (double)g[i] * exp(betas[k] * (double)(E - emax));
    Z += wgt;
    ZE += wgt * (double)E;
  }
  meanE[t] = ZE / Z;
}

// ---------------------------------------------------------------------------
// Batched kernels: block b works for job j with pre[j] <= b < pre[j+1], on the
// job's block b - pre[j]; the bodies are the one-job kernels', so a job's
// words are the same alone and in a batch.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int spb_job(const uint32_t *pre, int n, uint32_t v) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pre + mid) <= v) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The block's job descriptor is copied to SMEM once (SMEM cannot alias the
// job's global arrays, and a per-thread copy would go to the stack).
#define SPB_ITEM(KIND)                                        \
  __shared__ SpDev s_job;                                     \
  const uint32_t *pre_ = b.pre[KIND];                         \
  const int jb = spb_job(pre_, b.njobs, blockIdx.x);          \
  if (threadIdx.x == 0) s_job = b.jobs[jb];                   \
  __syncthreads();                                            \
  const SpDev &d = s_job;                                     \
  const int blk = (int)(blockIdx.x - __ldg(pre_ + jb));

__global__ void kb_sp_fill(const __grid_constant__ SpBatchDev b, int colour) {
  __shared__ SpDev d;
  if (threadIdx.x == 0) d = b.jobs[blockIdx.x];
  __syncthreads();
  if (colour < d.ncol) sp_fill_body(d);
}
__global__ void __launch_bounds__(512) kb_sp_pass(const __grid_constant__ SpBatchDev b, int colour) {
  extern __shared__ __align__(16) unsigned char smem[];
  SPB_ITEM(SPB_PASS0 + colour)
  sp_pass_any(d, colour, blk, smem);
}
__global__ void kb_sp_zero(const __grid_constant__ SpBatchDev b) {
  SPB_ITEM(SPB_ZERO)
  const long long i = (long long)blk * blockDim.x + threadIdx.x;
  if (i < (long long)d.nw * 64 * d.NR * d.NB) d.U2[i] = 0;
}
__global__ void __launch_bounds__(256) kb_sp_energy(const __grid_constant__ SpBatchDev b) {
  SPB_ITEM(SPB_ENERGY)
  sp_energy_body(d, (long long)blk * blockDim.x + threadIdx.x);
}
__global__ void __launch_bounds__(64) kb_sp_pt(const __grid_constant__ SpBatchDev b) {
  SPB_ITEM(SPB_PT)
  sp_pt_body(d, blk, threadIdx.x);
}
__global__ void __launch_bounds__(kPermRows) kb_sp_permute(const __grid_constant__ SpBatchDev b) {
  extern __shared__ u64 rows[];
  SPB_ITEM(SPB_PERMUTE)
  sp_permute_body(d, blk, rows);
}
__global__ void kb_sp_measure(const __grid_constant__ SpBatchDev b, int from_e) {
  SPB_ITEM(SPB_MEASURE)
  sp_measure_u2_body(d, (long long)blk * blockDim.x + threadIdx.x, from_e);
}
__global__ void kb_sp_pairs(const __grid_constant__ SpBatchDev b) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < b.njobs && b.jobs[j].nclust > 0) sp_pairs_body(b.jobs[j]);
}
__global__ void kb_sp_overlap(const __grid_constant__ SpBatchDev b, int g) {
  SPB_ITEM(SPB_OVL0 + g)
  sp_overlap_body(d, g, (long long)blk * blockDim.x + threadIdx.x);
}
__global__ void __launch_bounds__(1024, 1) kb_sp_cluster(const __grid_constant__ SpBatchDev b, int g) {
  extern __shared__ __align__(16) uint32_t sm[];
  SPB_ITEM(SPB_CL0 + g)
  sp_cluster_any(d, g, blk, reinterpret_cast<unsigned char *>(sm));
}
__global__ void kb_sp_flip(const __grid_constant__ SpBatchDev b, int g) {
  SPB_ITEM(SPB_FL0 + g)
  sp_flip_body(d, g, (long long)blk * blockDim.x + threadIdx.x);
}

size_t sp_cluster_smem(int V);

// Blocks of job d for each batched kernel kind (the one-job launch geometry).
void sp_batch_blocks(const SpDev &d, bool cluster, uint32_t out[SPB_COUNT]) {
  const long long G = (long long)d.NR * d.NB, nw = d.nw;
  for (int k = 0; k < SPB_COUNT; ++k) out[k] = 0;
  for (int c = 0; c < kSpBatchMaxColours && c < d.ncol; ++c) {
    const long long n = d.col_off[c + 1] - d.col_off[c];
    out[SPB_PASS0 + c] = d.pgrid ? (uint32_t)((n * G + 512LL * kItemsPerThread - 1) / (512LL * kItemsPerThread))
                                 : (uint32_t)((n + d.kt - 1) / d.kt);
  }
  out[SPB_ZERO] = out[SPB_MEASURE] = (uint32_t)((nw * 64 * G + 255) / 256);
  out[SPB_ENERGY] = (uint32_t)((nw * ((d.esites + d.echunk - 1) / d.echunk) * G + 255) / 256);
  out[SPB_PT] = (uint32_t)(nw * d.NR);
  out[SPB_PERMUTE] = (uint32_t)((nw * d.V * d.NR + kPermRows - 1) / kPermRows);
  if (cluster && d.nclust > 0) {
    const int ng = d.NR >= 4 ? 2 : 1;
    for (int g = 0; g < ng; ++g) {
      out[SPB_OVL0 + g] = out[SPB_FL0 + g] = (uint32_t)((nw * d.nclust * d.V + 255) / 256);
      out[SPB_CL0 + g] = (uint32_t)(nw * d.nclust * 8);
    }
  }
}

// Largest dynamic SMEM of a kernel: the 227 KB of a block less its static SMEM.
template <class K>
static cudaError_t max_dynamic_smem(K kernel) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024 - (int)fa.sharedSizeBytes);
}

cudaError_t sp_batch_setup() {
  cudaError_t e = max_dynamic_smem(kb_sp_pass);
  if (e == cudaSuccess) e = max_dynamic_smem(kb_sp_cluster);
  if (e == cudaSuccess) e = max_dynamic_smem(kb_sp_permute);
  return e;
}

// One sweep of every job: colour by colour, each job's counters advanced only
// for the colours it has.
cudaError_t sp_batch_sweep(const SpBatchDev &b, int ncol_max, cudaStream_t st) {
  for (int c = 0; c < ncol_max; ++c) {
    kb_sp_fill<<<b.njobs, 64, 0, st>>>(b, c);
    if (b.total[SPB_PASS0 + c]) kb_sp_pass<<<b.total[SPB_PASS0 + c], 512, b.pass_smem, st>>>(b, c);
  }
  return cudaGetLastError();
}

static void spb_energy(const SpBatchDev &b, cudaStream_t st) {
  kb_sp_zero<<<b.total[SPB_ZERO], 256, 0, st>>>(b);
  kb_sp_energy<<<b.total[SPB_ENERGY], 256, 0, st>>>(b);
}

cudaError_t sp_batch_tempering(const SpBatchDev &b, cudaStream_t st) {
  spb_energy(b, st);
  kb_sp_pt<<<b.total[SPB_PT], 64, 0, st>>>(b);
  kb_sp_permute<<<b.total[SPB_PERMUTE], kPermRows, b.perm_smem, st>>>(b);
  return cudaGetLastError();
}

cudaError_t sp_batch_houdayer(const SpBatchDev &b, cudaStream_t st) {
  kb_sp_pairs<<<(b.njobs + 127) / 128, 128, 0, st>>>(b);
  for (int g = 0; g < 2; ++g) {
    if (!b.total[SPB_CL0 + g]) continue;
    kb_sp_overlap<<<b.total[SPB_OVL0 + g], 256, 0, st>>>(b, g);
    kb_sp_cluster<<<b.total[SPB_CL0 + g], b.cluster_threads, b.cluster_smem, st>>>(b, g);
    kb_sp_flip<<<b.total[SPB_FL0 + g], 256, 0, st>>>(b, g);
  }
  return cudaGetLastError();
}

cudaError_t sp_batch_measure(const SpBatchDev &b, bool from_e, cudaStream_t st) {
  if (!from_e) spb_energy(b, st);
  kb_sp_measure<<<b.total[SPB_MEASURE], 256, 0, st>>>(b, from_e ? 1 : 0);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Persistent bin kernel: one cooperative launch runs whole bins of a set of
// jobs (one job, or a batch), every phase of the cadence -- colour passes
// with their counters, energies, tempering, permutes, Houdayer moves,
// measurements -- as a loop over the same packed (job, block) work list the
// batched kernels use, with a grid barrier between phases.  The bodies are
// the one-job kernels', in the same order, so the words are the same as with
// one launch per phase; what goes away is the launch and graph-node gap of
// every phase, which bounds jobs too small to fill the GPU.
// ---------------------------------------------------------------------------
constexpr int kPersistThreads = 512;
constexpr unsigned long long kBarrierWaitNs = 4000000000ull;  // 4 s

__device__ __forceinline__ unsigned long long sp_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid barrier of a cooperative launch (every block resident): arrivals are
// counted in *bar (zero at launch); the k-th barrier of the launch waits for
// k x gridDim.x arrivals.  A wait gives up after kBarrierWaitNs, or as soon
// as another block has given up, counts that in *err and returns false; the
// kernel then returns, so no block waits for ever and the host reports the
// failure.
__device__ bool sp_grid_sync(const SpPersistDev &p, unsigned &epoch) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ++epoch;
    const unsigned long long target = (unsigned long long)epoch * gridDim.x;
    __threadfence();
    atomicAdd(p.bar, 1ull);
    int ok = 1;
    const unsigned long long t0 = sp_globaltimer();
    for (;;) {
      unsigned long long v;
      asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p.bar) : "memory");
      if (v >= target) break;
      if (*(volatile int *)p.err) { ok = 0; break; }
      if (sp_globaltimer() - t0 > kBarrierWaitNs) { atomicAdd(p.err, 1); ok = 0; break; }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The blocks of one work-list kind whose bodies need a whole thread block.
#define SPP_BLOCKS(KIND, BODY)                                                        \
  for (uint32_t vb = blockIdx.x; vb < b.total[KIND]; vb += gridDim.x) {              \
    __syncthreads();                                                                  \
    if (threadIdx.x == 0) {                                                           \
      const int jb_ = spb_job(b.pre[KIND], b.njobs, vb);                              \
      s_job[0] = b.jobs[jb_];                                                         \
      s_blk[0] = (int)(vb - __ldg(b.pre[KIND] + jb_));                                \
    }                                                                                 \
    __syncthreads();                                                                  \
    const SpDev &d = s_job[0];                                                        \
    const int blk = s_blk[0];                                                         \
    BODY;                                                                             \
  }

// Kinds whose one-job blocks have SUB threads and no barrier: each thread
// block takes kPersistThreads / SUB of them at a time.
#define SPP_SUB(KIND, SUB, BODY)                                                      \
  for (uint32_t vb0 = blockIdx.x * (kPersistThreads / SUB); vb0 < b.total[KIND];      \
       vb0 += gridDim.x * (kPersistThreads / SUB)) {                                 \
    const int sub = threadIdx.x / SUB, ltid = threadIdx.x % SUB;                      \
    const uint32_t vb = vb0 + sub;                                                    \
    __syncthreads();                                                                  \
    if (ltid == 0 && vb < b.total[KIND]) {                                            \
      const int jb_ = spb_job(b.pre[KIND], b.njobs, vb);                              \
      s_job[sub] = b.jobs[jb_];                                                       \
      s_blk[sub] = (int)(vb - __ldg(b.pre[KIND] + jb_));                              \
    }                                                                                 \
    __syncthreads();                                                                  \
    if (vb < b.total[KIND]) {                                                         \
      const SpDev &d = s_job[sub];                                                    \
      const int blk = s_blk[sub];                                                     \
      BODY;                                                                           \
    }                                                                                 \
  }

#define SPP_SYNC() \
  if (!sp_grid_sync(p, epoch)) return

__global__ void __launch_bounds__(kPersistThreads, 1) k_sp_persist(const __grid_constant__ SpPersistDev p) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SpDev s_job[kPersistThreads / 64];
  __shared__ int s_blk[kPersistThreads / 64];
  const SpBatchDev &b = p.b;
  unsigned epoch = 0;
  auto energy = [&]() -> bool {
    SPP_SUB(SPB_ZERO, 256, {
      const long long i = (long long)blk * 256 + ltid;
      if (i < (long long)d.nw * 64 * d.NR * d.NB) d.U2[i] = 0;
    })
    if (!sp_grid_sync(p, epoch)) return false;
    SPP_SUB(SPB_ENERGY, 256, sp_energy_body(d, (long long)blk * 256 + ltid))
    return sp_grid_sync(p, epoch);
  };
  for (int it = 0; it < p.itmax; ++it) {
    for (int im = 0; im < p.mesfr; ++im) {
      for (int ih = 0; ih < p.houfr; ++ih) {
        for (int sw = 0; sw < p.ptfr; ++sw) {
          for (int c = 0; c < p.ncol_max; ++c) {
            for (int j = blockIdx.x; j < b.njobs; j += gridDim.x) {
              __syncthreads();
              if (threadIdx.x == 0) s_job[0] = b.jobs[j];
              __syncthreads();
              if (c < s_job[0].ncol) sp_fill_body(s_job[0]);
            }
            SPP_SYNC();
            SPP_BLOCKS(SPB_PASS0 + c, sp_pass_any(d, c, blk, smem))
            SPP_SYNC();
          }
        }
        if (!energy()) return;
        SPP_SUB(SPB_PT, 64, sp_pt_body(d, blk, ltid))
        SPP_SYNC();
        SPP_BLOCKS(SPB_PERMUTE, sp_permute_body(d, blk, reinterpret_cast<u64 *>(smem)))
        SPP_SYNC();
      }
      if (p.cluster) {
        for (int j = blockIdx.x * kPersistThreads + threadIdx.x; j < b.njobs; j += gridDim.x * kPersistThreads)
          if (b.jobs[j].nclust > 0) sp_pairs_body(b.jobs[j]);
        SPP_SYNC();
        for (int g = 0; g < 2; ++g) {
          if (!b.total[SPB_CL0 + g]) continue;
          SPP_SUB(SPB_OVL0 + g, 256, sp_overlap_body(d, g, (long long)blk * 256 + ltid))
          SPP_SYNC();
          SPP_BLOCKS(SPB_CL0 + g, sp_cluster_any(d, g, blk, smem))
          SPP_SYNC();
          SPP_SUB(SPB_FL0 + g, 256, sp_flip_body(d, g, (long long)blk * 256 + ltid))
          SPP_SYNC();
        }
      }
    }
    if (p.cluster && !energy()) return;
    SPP_SUB(SPB_MEASURE, 256, sp_measure_u2_body(d, (long long)blk * 256 + ltid, !p.cluster))
    SPP_SYNC();
  }
}

#undef SPP_SYNC
#undef SPP_SUB
#undef SPP_BLOCKS

// Blocks of a cooperative launch of k_sp_persist with `smem` bytes of dynamic
// SMEM: every block resident at once (one per SM, the kernel's registers and
// SMEM allowing), and no more than the largest phase has work for.
int sp_persist_grid(const SpBatchDev &b, size_t smem) {
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 0;
  if (cudaFuncSetAttribute(k_sp_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sp_persist, kPersistThreads, smem) != cudaSuccess ||
      per_sm < 1)
    return 0;
  uint32_t work = (uint32_t)b.njobs;
  for (int k = 0; k < SPB_COUNT; ++k) {
    const uint32_t sub = (k == SPB_PT) ? kPersistThreads / 64
                         : (k >= SPB_PASS0 && k <= SPB_PASS3) || k == SPB_PERMUTE || k == SPB_CL0 || k == SPB_CL1
                             ? 1 : kPersistThreads / 256;
    work = std::max(work, (b.total[k] + sub - 1) / sub);
  }
  return (int)std::min<uint32_t>(work, (uint32_t)(per_sm * nsm));
}

cudaError_t sp_launch_persist(const SpPersistDev &p, int grid, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(p.bar, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  void *args[] = {const_cast<SpPersistDev *>(&p)};
  return cudaLaunchCooperativeKernel((const void *)k_sp_persist, dim3(grid), dim3(kPersistThreads), args, smem, st);
}

// ---------------------------------------------------------------------------
// One-job kernels: the bodies above, one block per item
// ---------------------------------------------------------------------------
__global__ void k_sp_fill(const __grid_constant__ SpDev d) { sp_fill_body(d); }
// Pseudo-random overlap words (a 64-bit mix of the index) for timing the
// labelling on clusters of a random overlap; only the autotuner uses it.
__global__ void k_sp_noise(unsigned long long *Q, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long x = (unsigned long long)i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  x ^= x >> 31; x *= 0xBF58476D1CE4E5B9ull; x ^= x >> 29; x *= 0x94D049BB133111EBull; x ^= x >> 32;
  Q[i] = x;
}
__global__ void __launch_bounds__(512) k_sp_pass(const __grid_constant__ SpDev d, int off, int n) {
  extern __shared__ __align__(16) unsigned char smem[];
  sp_pass_body(d, off, n, blockIdx.x, smem);
}

__global__ void __launch_bounds__(512) k_sp_pass_items(const __grid_constant__ SpDev d, int off, int n) {
  extern __shared__ __align__(16) unsigned char smem[];
  sp_pass_items_body(d, off, n, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)n * d.NR * d.NB,
                     (long long)gridDim.x * blockDim.x, smem);
}
__global__ void __launch_bounds__(256) k_sp_energy(const __grid_constant__ SpDev d) {
  sp_energy_body(d, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void __launch_bounds__(64) k_sp_pt(const __grid_constant__ SpDev d) { sp_pt_body(d, blockIdx.x, threadIdx.x); }
__global__ void __launch_bounds__(kPermRows) k_sp_permute(const __grid_constant__ SpDev d) {
  extern __shared__ u64 rows[];
  sp_permute_body(d, blockIdx.x, rows);
}
__global__ void k_sp_pairs(const __grid_constant__ SpDev d) {
  if (threadIdx.x == 0) sp_pairs_body(d);
}
__global__ void k_sp_overlap(const __grid_constant__ SpDev d, int g) {
  sp_overlap_body(d, g, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void __launch_bounds__(1024, 1) k_sp_cluster(const __grid_constant__ SpDev d, int g) {
  extern __shared__ __align__(16) uint32_t sm[];
  sp_cluster_any(d, g, blockIdx.x, reinterpret_cast<unsigned char *>(sm));
}
__global__ void __launch_bounds__(1024, 1) k_sp_slab8(const __grid_constant__ SpDev d) {
  extern __shared__ __align__(16) unsigned char sm8[];
  sp_slab8_body(d, blockIdx.y, blockIdx.x, sm8);
}
__global__ void k_sp_slab_merge(const __grid_constant__ SpDev d) {
  sp_slab_merge_body(d, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_sp_slab_roots(const __grid_constant__ SpDev d, int g) {
  sp_slab_roots_body(d, g, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_sp_slab_flip(const __grid_constant__ SpDev d) {
  sp_slab_flip_body(d, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_sp_flip(const __grid_constant__ SpDev d, int g) {
  sp_flip_body(d, g, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_sp_measure_u2(const __grid_constant__ SpDev d, int from_e) {
  sp_measure_u2_body(d, (long long)blockIdx.x * blockDim.x + threadIdx.x, from_e);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
size_t sp_cluster_smem(int V);

size_t sp_sweep_smem(int NB, int NR, int kt) {
  return (size_t)NB * 256 * 10 + (size_t)3 * NB * kt * NR * 8 + (size_t)kt * 7 * 4;
}
size_t sp_items_smem(int NB) { return (size_t)NB * kPre11Stride; }

// Grid of the per-item pass: every CTA resident at once (the kernel's
// registers and the threshold tables' SMEM allowing); 0 if none fits.
int sp_items_grid(int NB) {
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sp_pass_items, 512, sp_items_smem(NB)) != cudaSuccess)
    return 0;
  return per_sm * nsm;
}

// Tile width: the smallest power of two whose random triples (NB x kt x NR)
// fill half of the CTA's 512 threads -- narrower tiles leave the CTA staging
// every threshold table for a few words -- then doubled while two tiles per
// SM remain and SMEM fits (large jobs amortise the staging over more sites).
int sp_kt(int NB, int NR, int nsites_colour) {
  int kt = 1;
  while (kt < 64 && NB * kt * NR < 256) kt <<= 1;
  const size_t lim = 227 * 1024 - 512;  // room for the batched kernels' static SMEM
  while (kt > 1 && sp_sweep_smem(NB, NR, kt) > lim) kt >>= 1;
  if (sp_sweep_smem(NB, NR, kt) > lim) return 0;
  while (kt < 64 && sp_sweep_smem(NB, NR, 2 * kt) <= lim && (nsites_colour + 2 * kt - 1) / (2 * kt) >= 2 * 152)
    kt <<= 1;
  return kt;
}

cudaError_t sp_setup() {
  cudaError_t e = cudaFuncSetAttribute(k_sp_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sp_pass_items, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_sp_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)std::max(sp_cluster_smem(kSpClusterMaxV),
                                           std::max(sp_cluster_smem(kSpCluster4MaxV), sp_cluster_smem(kSpCluster8MaxV))));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_sp_permute, cudaFuncAttributeMaxDynamicSharedMemorySize, kPermRows * 65 * 8);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_sp_slab8, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp_cluster_smem(kSpCluster8MaxV));
  return e;
}

cudaError_t sp_launch_pass(const SpDev &d, int colour, int off, int n, cudaStream_t st) {
  k_sp_fill<<<1, 64, 0, st>>>(d);
  (void)colour;
  if (n > 0 && d.pgrid > 0) {
    const long long blocks = ((long long)n * d.NR * d.NB + 511) / 512;
    k_sp_pass_items<<<(unsigned)std::min<long long>(blocks, d.pgrid), 512, sp_items_smem(d.NB), st>>>(d, off, n);
  } else if (n > 0) {
    const int grid = (n + d.kt - 1) / d.kt;
    k_sp_pass<<<grid, 512, sp_sweep_smem(d.NB, d.NR, d.kt), st>>>(d, off, n);
  }
  return cudaGetLastError();
}

cudaError_t sp_launch_energy(const SpDev &d, cudaStream_t st) {
  const int G = d.NR * d.NB;
  cudaError_t e = cudaMemsetAsync(d.U2, 0, sizeof(int32_t) * (size_t)d.nw * 64 * G, st);
  if (e != cudaSuccess) return e;
  const long long n = (long long)d.nw * ((d.esites + d.echunk - 1) / d.echunk) * G;
  k_sp_energy<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d);
  return cudaGetLastError();
}

cudaError_t sp_launch_pt(const SpDev &d, cudaStream_t st) {
  k_sp_pt<<<d.nw * d.NR, 64, 0, st>>>(d);
  return cudaGetLastError();
}

cudaError_t sp_launch_permute(const SpDev &d, cudaStream_t st) {
  const long long n = (long long)d.nw * d.V * d.NR;
  k_sp_permute<<<(unsigned)((n + kPermRows - 1) / kPermRows), kPermRows, (size_t)kPermRows * (d.NB | 1) * 8, st>>>(d);
  return cudaGetLastError();
}


size_t sp_cluster_smem(int V) {
  return V <= kSpCluster8MaxV ? (size_t)V * 26 : V <= kSpCluster4MaxV ? (size_t)V * 22 : V <= kSpClusterMaxV ? (size_t)V * 7 : 0;
}

// Block size of the cluster labelling: 1024 threads, 256 for lattices of
// at most 2048 sites (256 threads measured 20 % slower on 6912 sites, 512 the
// same as 1024).
int sp_cluster_threads(int V) { return V <= 2048 ? 256 : 1024; }

// Planes per slab of the slab labelling of lattices above kSpClusterMaxV
// sites: as many whole planes as the 8-sample SMEM labelling takes; 0 (the
// one-CTA labelling in global scratch) when a plane alone is too large or
// the labels of every (word, slot, group) would pass 4 GB.
int sp_slab_planes(int L, int Lz, int nw, int nclust) {
  const long long L2 = (long long)L * L, V = L2 * Lz;
  if (V <= kSpClusterMaxV || L2 > kSpCluster8MaxV) return 0;
  if ((long long)nw * nclust * 8 * V * 33 > (4ll << 30)) return 0;
  return (int)std::min<long long>(Lz, kSpCluster8MaxV / L2);
}

cudaError_t sp_launch_houdayer(const SpDev &d, cudaStream_t st) {
  k_sp_pairs<<<1, 32, 0, st>>>(d);
  const int ng = d.NR >= 4 ? 2 : 1;
  for (int g = 0; g < ng; ++g) {
    const long long n = (long long)d.nw * d.nclust * d.V;
    k_sp_overlap<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d, g);
    if (d.slabD > 0) {
      const int L2 = d.L * d.L, nslab = (d.Lz + d.slabD - 1) / d.slabD, nunits = d.nw * d.nclust * 8;
      const long long nu = (long long)nunits * d.V;
      k_sp_slab8<<<dim3((unsigned)nslab, (unsigned)nunits), 1024, sp_cluster_smem(d.slabD * L2), st>>>(d);
      k_sp_slab_merge<<<(unsigned)((nu + 255) / 256), 256, 0, st>>>(d);
      k_sp_slab_roots<<<(unsigned)((nu + 255) / 256), 256, 0, st>>>(d, g);
      k_sp_slab_flip<<<(unsigned)((nu + 255) / 256), 256, 0, st>>>(d);
    } else {
      k_sp_cluster<<<(unsigned)(d.nw * d.nclust * 8), d.cthreads, sp_cluster_smem(d.V), st>>>(d, g);
    }
    k_sp_flip<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d, g);
  }
  return cudaGetLastError();
}

cudaError_t sp_launch_measure_u2(const SpDev &d, bool from_e, cudaStream_t st) {
  const long long n = (long long)d.nw * 64 * d.NR * d.NB;
  k_sp_measure_u2<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d, from_e ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t sp_launch_dos(const SpDev &d, cudaStream_t st) {
  const int nlow = std::min(kDosLow, d.V - 1);
  const int npre = d.V - 1 - nlow;
  const unsigned long long nthreads = 1ull << npre;
  const dim3 grid((unsigned)((nthreads + 255) / 256), (unsigned)(d.nw * 64));
  k_sp_dos<<<grid, 256, 0, st>>>(d, npre);
  return cudaGetLastError();
}

cudaError_t sp_launch_exact(const SpDev &d, const double *betas, int nbeta, double *meanE, cudaStream_t st) {
  const int n = d.nw * 64 * nbeta;
  k_sp_exact<<<(n + 127) / 128, 128, 0, st>>>(d, betas, nbeta, meanE);
  return cudaGetLastError();
}

}  // namespace eagb

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace eagb;

namespace {
int spfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  set_last_error(buf);
  return code;
}
#define SCU(call)                                                                             \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return spfail(EA_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)
}  // namespace

struct ea_sp {
  ea_sp_geom geom{};
  SpGraph g;
  int device = 0;
  cudaStream_t st = nullptr;
  SpDev d{};
  std::vector<void *> owned;
  std::vector<int32_t> expoff;
  double *exptab = nullptr;
  bool have_temps = false;
  // one iteration of the bin cadence, replayed as a CUDA graph
  cudaGraphExec_t it_graph = nullptr;
  ea_cadence it_cad{};
  int q_cap = 0;  // slots the overlap buffer holds
  SpDev it_dev{};  // the descriptor the graph was captured with
  int last_itmax = 0;  // iterations of the last bin (alone or batched)
  // persistent bin kernel of the job alone (EA_BIN_*)
  int bin_mode = EA_BIN_AUTO;
  SpDev *p_jobs = nullptr;            // [1] descriptor of the work list
  uint32_t *p_pre = nullptr;          // [SPB_COUNT][2] block prefix sums
  unsigned long long *p_bar = nullptr;
  int *p_err = nullptr;
  SpDev p_up{};                       // descriptor last uploaded
  bool p_valid = false;
  // resident bin kernel (EA_BIN_RESIDENT): plan for the descriptor r_dev,
  // Philox counters and random words of one launch's passes
  SpResPlan r_plan{};
  SpDev r_dev{};
  int r_state = 0;                    // 0: not planned, 1: eligible, 2: not eligible
  uint4 *r_ctrs = nullptr;
  unsigned long long *r_R = nullptr, *r_X = nullptr;
  size_t r_cap_pass = 0, r_cap_sweep = 0, r_cap_pt = 0;
  bool pair_energy = false;           // see sp_pair_energy
};

namespace {
template <class T>
int sp_own(ea_sp *c, T *&p, size_t n) {
  cudaError_t e = cudaMalloc((void **)&p, sizeof(T) * (n ? n : 1));
  if (e != cudaSuccess) return spfail(EA_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", sizeof(T) * n, cudaGetErrorString(e));
  c->owned.push_back((void *)p);
  cudaMemsetAsync(p, 0, sizeof(T) * (n ? n : 1), c->st);
  return EA_OK;
}

bool geom_ok(const ea_sp_geom *g) {
  return g && g->nbetas >= 2 && g->nbetas <= 64 && g->nrep >= 1 && g->nrep <= 64 && g->nwords >= 1 &&
         g->nwords <= (1 << 20);
}
}  // namespace

extern "C" {

int ea_sp_graph(int32_t L, int32_t Lz, int32_t bc, int32_t *nb, int32_t *mate, uint8_t *colour, int32_t *ncol) {
  SpGraph g;
  if (!sp_graph(L, Lz, bc, g)) return spfail(EA_ERR_ARG, "tube %d x %d x %d (bc %d) not supported", L, L, Lz, bc);
  if (nb) std::memcpy(nb, g.nb.data(), g.nb.size() * 4);
  if (mate) std::memcpy(mate, g.mate.data(), g.mate.size() * 4);
  if (colour) std::memcpy(colour, g.colour.data(), g.colour.size());
  if (ncol) *ncol = g.ncol;
  return EA_OK;
}

int ea_sp_host_init(const ea_sp_geom *gp, uint64_t seed_J, uint64_t seed_u, uint64_t *J, uint64_t *S) {
  SpGraph g;
  if (!geom_ok(gp) || !sp_graph(gp->L, gp->Lz, gp->bc, g)) return spfail(EA_ERR_ARG, "bad sample-packed geometry");
  if (J) sp_couplings(g, gp->nwords, seed_J, J);
  if (S) sp_spins(g, gp->nwords, gp->nrep, gp->nbetas, seed_u, S);
  return EA_OK;
}

int ea_sp_presearch11(const uint64_t *cum, uint8_t *pre) {
  if (!cum || !pre) return spfail(EA_ERR_ARG, "null argument");
  if (cum[255] != ~0ULL) return spfail(EA_ERR_ARG, "threshold 255 is not 2^64-1");
  presearch11(cum, pre);
  return EA_OK;
}

int ea_sp_create(const ea_sp_geom *gp, int32_t device, ea_sp **out) {
  if (!gp || !out) return spfail(EA_ERR_ARG, "null argument");
  if (!geom_ok(gp)) return spfail(EA_ERR_ARG, "2 <= nbetas <= 64, 1 <= nrep <= 64, nwords >= 1");
  ea_sp *c = new ea_sp();
  c->geom = *gp;
  if (!sp_graph(gp->L, gp->Lz, gp->bc, c->g)) {
    delete c;
    return spfail(EA_ERR_ARG, "tube %d x %d x %d (bc %d) not supported", gp->L, gp->L, gp->Lz, gp->bc);
  }
  const SpGraph &g = c->g;
  SpDev &d = c->d;
  d.L = g.L; d.Lz = g.Lz; d.V = g.V; d.bc = g.bc; d.NB = gp->nbetas; d.NR = gp->nrep; d.nw = gp->nwords;
  d.ncol = g.ncol;
  int maxc = 0;
  for (int k = 0; k < g.ncol; ++k) maxc = std::max(maxc, g.col_off[k + 1] - g.col_off[k]);
  d.kt = sp_kt(d.NB, d.NR, maxc);
  d.cthreads = sp_cluster_threads(d.V);
  d.esites = d.V;
  d.epair = 0;
  d.echunk = sp_energy_chunk(d);
  for (int k = 0; k <= g.ncol && k < 9; ++k) d.col_off[k] = g.col_off[k];
  if (!d.kt) { delete c; return spfail(EA_ERR_ARG, "NB=%d x NR=%d does not fit in shared memory", d.NB, d.NR); }
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = sp_setup();
  if (e == cudaSuccess) e = sp_res_setup();
  if (e != cudaSuccess) { delete c; return spfail(EA_ERR_CUDA, "set-up: %s", cudaGetErrorString(e)); }
  const size_t G = (size_t)d.NR * d.NB, V = g.V, nw = d.nw;
  int rc;
#define SOWN(p, n) if ((rc = sp_own(c, p, n)) != EA_OK) { ea_sp_destroy(c); return rc; }
  { int32_t *p; SOWN(p, V * 6); d.nb = p; }
  { int32_t *p; SOWN(p, V); d.col_sites = p; }
  SOWN(d.S, nw * V * G);
  { unsigned long long *p; SOWN(p, nw * V * 6); d.J = p; }
  { unsigned long long *p; SOWN(p, (size_t)d.NB * 256); d.cum = p; }
  { uint16_t *p; SOWN(p, (size_t)d.NB * 256); d.pre = p; }
  { uint8_t *p; SOWN(p, (size_t)d.NB * kPre11Stride); d.pre11 = p; }
  SOWN(d.ctr, (size_t)d.NR);
  { uint32_t *p; SOWN(p, (size_t)d.NR); d.keys = p; }
  SOWN(d.prc, (size_t)d.NR);
  SOWN(d.xo, (size_t)d.NR);
  SOWN(d.iter, 1);
  SOWN(d.U2, nw * 64 * G);
  SOWN(d.E, nw * 64 * G);
  SOWN(d.perm, nw * 64 * G);
  SOWN(d.acc, nw * 64 * d.NR * (d.NB - 1));
  SOWN(d.M, nw * d.NR * (d.NB - 1));
  { double *p; SOWN(p, (size_t)d.NB); d.betas = p; }
  { int32_t *p; SOWN(p, (size_t)d.NB); d.expoff = p; }
  SOWN(d.ptstep, 1);
  SOWN(d.avgE, nw * 64 * G);
  SOWN(d.rc, 1);
  SOWN(d.pairs, 4);
  SOWN(d.move, 1);
#undef SOWN
  SCU(cudaMemcpyAsync((void *)d.nb, g.nb.data(), V * 6 * 4, cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync((void *)d.col_sites, g.col_sites.data(), V * 4, cudaMemcpyHostToDevice, c->st));
  // identity slot -> configuration map
  std::vector<uint8_t> perm(nw * 64 * G);
  for (size_t i = 0; i < perm.size(); ++i) perm[i] = (uint8_t)(i % d.NB);
  SCU(cudaMemcpyAsync(d.perm, perm.data(), perm.size(), cudaMemcpyHostToDevice, c->st));
  SCU(cudaStreamSynchronize(c->st));
  // one-word jobs take the per-item pass: measured faster than every tile
  // width on one word (L=6 to 24, 12 to 32 temperatures); many words share
  // each tile's random words and keep the tiles
  if (nw == 1) d.pgrid = sp_items_grid(d.NB);
  *out = c;
  return EA_OK;
}

int ea_sp_destroy(ea_sp *c) {
  if (!c) return EA_OK;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  for (void *p : c->owned) cudaFree(p);
  if (c->exptab) cudaFree(c->exptab);
  if (c->d.dos) cudaFree(c->d.dos);
  if (c->d.Q) cudaFree(c->d.Q);
  if (c->d.cscratch) cudaFree(c->d.cscratch);
  if (c->d.slab_lab) cudaFree(c->d.slab_lab);
  if (c->d.slab_coin) cudaFree(c->d.slab_coin);
  if (c->it_graph) cudaGraphExecDestroy(c->it_graph);
  if (c->p_jobs) cudaFree(c->p_jobs);
  if (c->p_pre) cudaFree(c->p_pre);
  if (c->p_bar) cudaFree(c->p_bar);
  if (c->p_err) cudaFree(c->p_err);
  if (c->r_ctrs) cudaFree(c->r_ctrs);
  if (c->r_R) cudaFree(c->r_R);
  if (c->r_X) cudaFree(c->r_X);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return EA_OK;
}

// The job's device view and stream, for the analysis entry points of
// sp_analysis.cu (current device set to the job's).
int ea_sp_device_view(ea_sp *c, SpDev *d, cudaStream_t *st) {
  if (!c || !d || !st) return spfail(EA_ERR_ARG, "null argument");
  SCU(cudaSetDevice(c->device));
  *d = c->d;
  *st = c->st;
  return EA_OK;
}

int ea_sp_info(const ea_sp *c, int32_t *ncol, int32_t *tile) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  if (ncol) *ncol = c->d.ncol;
  if (tile) *tile = c->d.pgrid ? 0 : c->d.kt;
  return EA_OK;
}

int ea_sp_stream(ea_sp *c, void **stream) {
  if (!c || !stream) return spfail(EA_ERR_ARG, "null argument");
  *stream = (void *)c->st;
  return EA_OK;
}

// After a synchronisation: did a persistent bin kernel give up on a barrier?
static int sp_check_persist(int *d_err, cudaStream_t st) {
  if (!d_err) return EA_OK;
  int err = 0;
  SCU(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SCU(cudaStreamSynchronize(st));
  if (err) {
    SCU(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    return spfail(EA_ERR_CUDA, "persistent bin kernel: a grid barrier wait gave up (%d blocks); the bin is incomplete", err);
  }
  return EA_OK;
}

int ea_sp_sync(ea_sp *c) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  SCU(cudaSetDevice(c->device));
  SCU(cudaStreamSynchronize(c->st));
  return sp_check_persist(c->p_err, c->st);
}

int ea_sp_set_tile(ea_sp *c, int32_t tile) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  SCU(cudaSetDevice(c->device));
  SpDev &d = c->d;
  if (tile == 0) {
    const int pg = sp_items_grid(d.NB);
    if (!pg) return spfail(EA_ERR_ARG, "the per-item pass does not fit NB=%d", d.NB);
    d.pgrid = pg;
    return EA_OK;
  }
  if (tile < 1 || tile > 64 || sp_sweep_smem(d.NB, d.NR, tile) > 227 * 1024 - 512)
    return spfail(EA_ERR_ARG, "tile %d: 1..64 sites whose tables fit in shared memory", tile);
  d.kt = tile;
  d.pgrid = 0;
  return EA_OK;
}

int ea_sp_set_bin_kernel(ea_sp *c, int32_t mode) {
  if (!c || mode < EA_BIN_AUTO || mode > EA_BIN_RESIDENT) return spfail(EA_ERR_ARG, "bad bin-kernel mode");
  c->bin_mode = mode;
  return EA_OK;
}

int ea_sp_set_temperatures(ea_sp *c, const double *betas, const uint64_t *cum) {
  if (!c || !betas || !cum) return spfail(EA_ERR_ARG, "null argument");
  const int NB = c->d.NB;
  for (int i = 0; i + 1 < NB; ++i)
    if (betas[i] < betas[i + 1]) return spfail(EA_ERR_ARG, "betas must be sorted from largest to smallest");
  std::vector<uint16_t> pre((size_t)NB * 256);
  std::vector<uint8_t> pre11((size_t)NB * kPre11Stride);
  for (int b = 0; b < NB; ++b) {
    if (cum[(size_t)b * 256 + 255] != ~0ULL) return spfail(EA_ERR_ARG, "threshold 255 of beta %d is not 2^64-1", b);
    presearch8(cum + (size_t)b * 256, pre.data() + (size_t)b * 256);
    presearch11(cum + (size_t)b * 256, pre11.data() + (size_t)b * kPre11Stride);
  }
  std::vector<double> tab;
  pt_exp_table(betas, NB, tab, c->expoff);
  SCU(cudaSetDevice(c->device));
  SCU(cudaStreamSynchronize(c->st));
  if (c->exptab) cudaFree(c->exptab);
  c->exptab = nullptr;
  SCU(cudaMalloc((void **)&c->exptab, sizeof(double) * std::max<size_t>(1, tab.size())));
  SCU(cudaMemcpyAsync(c->exptab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync((void *)c->d.cum, cum, sizeof(uint64_t) * 256 * NB, cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync((void *)c->d.pre, pre.data(), pre.size() * 2, cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync((void *)c->d.pre11, pre11.data(), pre11.size(), cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync((void *)c->d.betas, betas, sizeof(double) * NB, cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync((void *)c->d.expoff, c->expoff.data(), sizeof(int32_t) * NB, cudaMemcpyHostToDevice, c->st));
  SCU(cudaStreamSynchronize(c->st));
  c->d.exptab = c->exptab;
  c->have_temps = true;
  c->r_state = 0;  // the resident plan stages the exp table: plan again
  return EA_OK;
}

int ea_sp_set_generators(ea_sp *c, const ea_generators *gen, uint64_t pt_seed) {
  if (!c || !gen) return spfail(EA_ERR_ARG, "null argument");
  const int NR = c->d.NR;
  SCU(cudaSetDevice(c->device));
  SCU(cudaMemcpyAsync(c->d.prc, gen->prc, sizeof(ea_hq) * NR, cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync(c->d.xo, gen->xo, sizeof(ea_xoshiro) * NR, cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync((void *)c->d.keys, gen->keys, sizeof(uint32_t) * NR, cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync(c->d.rc, &gen->rc, sizeof(ea_hq), cudaMemcpyHostToDevice, c->st));
  SCU(cudaStreamSynchronize(c->st));
  c->d.pt_seed = pt_seed;
  return EA_OK;
}

int ea_sp_get_generators(ea_sp *c, ea_generators *gen) {
  if (!c || !gen) return spfail(EA_ERR_ARG, "null argument");
  const int NR = c->d.NR;
  std::memset(gen, 0, sizeof(*gen));
  SCU(cudaSetDevice(c->device));
  SCU(cudaMemcpyAsync(gen->prc, c->d.prc, sizeof(ea_hq) * NR, cudaMemcpyDeviceToHost, c->st));
  SCU(cudaMemcpyAsync(gen->xo, c->d.xo, sizeof(ea_xoshiro) * NR, cudaMemcpyDeviceToHost, c->st));
  SCU(cudaMemcpyAsync(gen->keys, c->d.keys, sizeof(uint32_t) * NR, cudaMemcpyDeviceToHost, c->st));
  SCU(cudaMemcpyAsync(&gen->rc, c->d.rc, sizeof(ea_hq), cudaMemcpyDeviceToHost, c->st));
  SCU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

int ea_sp_init(ea_sp *c, const uint64_t seeds[4], uint32_t jobid) {
  if (!c || !seeds) return spfail(EA_ERR_ARG, "null argument");
  const SpDev &d = c->d;
  const size_t G = (size_t)d.NR * d.NB;
  std::vector<uint64_t> J((size_t)d.nw * d.V * 6), S((size_t)d.nw * d.V * G);
  sp_couplings(c->g, d.nw, seeds[0], J.data());
  sp_spins(c->g, d.nw, d.NR, d.NB, seeds[1], S.data());
  // Metropolis generators per replica as Init_Random seeds them
  // (random_generator.cu:94-158, 203-241), from seed_MC
  std::vector<uint64_t> sMC(d.NR);
  seeds_from_one(seeds[2], sMC.data(), d.NR);
  std::vector<ea_generators> gen(1);
  std::memset(gen.data(), 0, sizeof(ea_generators));
  for (int r = 0; r < d.NR; ++r) init_generators(sMC[r], gen[0].prc[r], gen[0].xo[r], gen[0].keys[r]);
  // replica-pair generator of the cluster moves, a Parisi-Rapuano stream
  // seeded from seed_PT as Init_Rand_HQ_64bits seeds one
  hq_seed(gen[0].rc, seeds[3]);
  int rc = ea_sp_set_couplings(c, J.data());
  if (!rc) rc = ea_sp_set_spins(c, S.data());
  if (!rc) rc = ea_sp_set_generators(c, gen.data(), seeds[3]);
  if (!rc) rc = ea_sp_set_counter(c, 0, 0, jobid);
  return rc;
}

int ea_sp_set_spins(ea_sp *c, const uint64_t *S) {
  if (!c || !S) return spfail(EA_ERR_ARG, "null argument");
  SCU(cudaSetDevice(c->device));
  SCU(cudaMemcpyAsync(c->d.S, S, (size_t)c->d.nw * c->d.V * c->d.NR * c->d.NB * 8, cudaMemcpyHostToDevice, c->st));
  SCU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

int ea_sp_get_spins(ea_sp *c, uint64_t *S) {
  if (!c || !S) return spfail(EA_ERR_ARG, "null argument");
  SCU(cudaSetDevice(c->device));
  SCU(cudaMemcpyAsync(S, c->d.S, (size_t)c->d.nw * c->d.V * c->d.NR * c->d.NB * 8, cudaMemcpyDeviceToHost, c->st));
  SCU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

// Whether U2 equals twice the unsatisfied half-edges of the colour-1 sites:
// two colours, every half-edge's mate at the other end of its bond (on the
// other colour), and both ends holding the same coupling word.
static bool sp_pair_energy(const SpGraph &g, int nw, const uint64_t *J) {
  if (g.ncol != 2) return false;
  for (int h = 0; h < g.V * 6; ++h) {
    const int i = h / 6, m = g.mate[h], j = m / 6;
    if (m < 0 || m >= g.V * 6 || g.nb[h] != j || g.nb[m] != i || g.mate[m] != h || g.colour[i] == g.colour[j])
      return false;
    for (int w = 0; w < nw; ++w)
      if (J[(size_t)w * g.V * 6 + h] != J[(size_t)w * g.V * 6 + m]) return false;
  }
  return true;
}

int ea_sp_set_couplings(ea_sp *c, const uint64_t *J) {
  if (!c || !J) return spfail(EA_ERR_ARG, "null argument");
  SCU(cudaSetDevice(c->device));
  SCU(cudaMemcpyAsync((void *)c->d.J, J, (size_t)c->d.nw * c->d.V * 6 * 8, cudaMemcpyHostToDevice, c->st));
  SCU(cudaStreamSynchronize(c->st));
  c->pair_energy = sp_pair_energy(c->g, c->d.nw, J);
  c->d.epair = c->pair_energy ? 1 : 0;
  c->d.esites = c->pair_energy ? c->g.col_off[2] - c->g.col_off[1] : c->d.V;
  c->d.echunk = sp_energy_chunk(c->d);
  return EA_OK;
}

int ea_sp_set_counter(ea_sp *c, int64_t iter, uint64_t ptstep, uint32_t jobid) {
  if (!c || jobid >= (1u << 14)) return spfail(EA_ERR_ARG, "job id < 2^14");
  SCU(cudaSetDevice(c->device));
  c->d.jobid = jobid;
  SCU(cudaMemcpyAsync(c->d.iter, &iter, 8, cudaMemcpyHostToDevice, c->st));
  SCU(cudaMemcpyAsync(c->d.ptstep, &ptstep, 8, cudaMemcpyHostToDevice, c->st));
  SCU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

int ea_sp_get_counter(ea_sp *c, int64_t *iter, uint64_t *ptstep) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  SCU(cudaSetDevice(c->device));
  int64_t it = 0;
  uint64_t ps = 0;
  SCU(cudaMemcpyAsync(&it, c->d.iter, 8, cudaMemcpyDeviceToHost, c->st));
  SCU(cudaMemcpyAsync(&ps, c->d.ptstep, 8, cudaMemcpyDeviceToHost, c->st));
  SCU(cudaStreamSynchronize(c->st));
  if (iter) *iter = it;
  if (ptstep) *ptstep = ps;
  return EA_OK;
}

// Autotuner: times the launch shapes that leave the results unchanged -- the
// colour pass's tile width, the energy count's sites per thread and the
// labelling's block size -- on the job itself and keeps the fastest.  What
// the timing runs change (spin words, pass counter, Philox counters, the two
// generators feeding them, the energy counts) is copied aside on the device
// first and put back after; the labelling runs on pseudo-random overlap words
// in the job's overlap buffer, which every move rewrites.
static int sp_sweeps(ea_sp *c, int n);
static int sp_cluster_prepare(ea_sp *c, int &nclust);

int ea_sp_autotune(ea_sp *c, int32_t *tile, int32_t *echunk, int32_t *cthreads) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  if (!c->have_temps) return spfail(EA_ERR_STATE, "temperatures not set");
  SCU(cudaSetDevice(c->device));
  SpDev &d = c->d;
  const size_t G = (size_t)d.NR * d.NB;
  struct Part { void *p; size_t n; };
  const Part parts[] = {{d.S, (size_t)d.nw * d.V * G * 8}, {d.iter, 8}, {d.ctr, sizeof(uint4) * d.NR},
                        {d.prc, sizeof(ea_hq) * d.NR}, {d.xo, sizeof(ea_xoshiro) * d.NR},
                        {d.U2, (size_t)d.nw * 64 * G * 4}};
  size_t total = 0;
  for (const Part &q : parts) total += (q.n + 255) & ~(size_t)255;
  char *save = nullptr;
  SCU(cudaMalloc((void **)&save, total));
  size_t off = 0;
  for (const Part &q : parts) {
    SCU(cudaMemcpyAsync(save + off, q.p, q.n, cudaMemcpyDeviceToDevice, c->st));
    off += (q.n + 255) & ~(size_t)255;
  }
  cudaEvent_t e0, e1;
  SCU(cudaEventCreate(&e0));
  SCU(cudaEventCreate(&e1));
  auto timed = [&](auto &&body) -> float {
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {  // the first run warms up
      cudaEventRecord(e0, c->st);
      body();
      cudaEventRecord(e1, c->st);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep) best = std::min(best, ms);
    }
    return cudaGetLastError() == cudaSuccess ? best : 1e30f;
  };
  int maxc = 0;
  for (int k = 0; k < d.ncol; ++k) maxc = std::max(maxc, d.col_off[k + 1] - d.col_off[k]);
  // colour pass: the heuristic's tile width and its neighbours that fit in
  // SMEM, and the per-item pass
  const int kt0 = d.kt, pg0 = d.pgrid;
  int best_kt = kt0, best_pg = pg0;
  float best = 1e30f;
  d.pgrid = 0;
  for (int kt : {kt0 / 2, kt0, kt0 * 2, kt0 * 4}) {
    if (kt < 1 || kt > 64 || sp_sweep_smem(d.NB, d.NR, kt) > 227 * 1024 - 512) continue;
    if ((maxc + kt - 1) / kt < 1) continue;
    d.kt = kt;
    const float ms = timed([&] { sp_sweeps(c, 2); });
    if (ms < best) { best = ms; best_kt = kt; best_pg = 0; }
  }
  d.kt = best_kt;
  if (const int pg = sp_items_grid(d.NB)) {
    d.pgrid = pg;
    const float ms = timed([&] { sp_sweeps(c, 2); });
    if (ms < best) { best = ms; best_pg = pg; }
  }
  d.pgrid = best_pg;
  // sites per thread of the energy count
  const int ec0 = d.echunk;
  int best_ec = ec0;
  best = 1e30f;
  for (int ec : {ec0 / 4, ec0 / 2, ec0, ec0 * 2, ec0 * 4}) {
    if (ec < 1 || ec > 256) continue;
    d.echunk = ec;
    const float ms = timed([&] { sp_launch_energy(d, c->st); });
    if (ms < best) { best = ms; best_ec = ec; }
  }
  d.echunk = best_ec;
  // block size of the labelling (lattices labelled in SMEM)
  int best_ct = d.cthreads;
  if (d.V <= kSpClusterMaxV) {
    int nclust = 0;
    int rc = sp_cluster_prepare(c, nclust);
    if (rc) { cudaFree(save); return rc; }
    const long long nq = (long long)d.nw * d.nclust * d.V;
    best = 1e30f;
    for (int ct : {256, 512, 1024}) {
      const float ms = timed([&] {
        k_sp_noise<<<(unsigned)((nq + 255) / 256), 256, 0, c->st>>>(d.Q, nq);
        k_sp_cluster<<<(unsigned)(d.nw * d.nclust * 8), ct, sp_cluster_smem(d.V), c->st>>>(d, 0);
      });
      if (ms < best) { best = ms; best_ct = ct; }
    }
  }
  d.cthreads = best_ct;
  off = 0;
  for (const Part &q : parts) {
    cudaMemcpyAsync(q.p, save + off, q.n, cudaMemcpyDeviceToDevice, c->st);
    off += (q.n + 255) & ~(size_t)255;
  }
  const cudaError_t e = cudaStreamSynchronize(c->st);
  cudaFree(save);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  SCU(e);
  if (tile) *tile = d.pgrid ? 0 : d.kt;
  if (echunk) *echunk = d.echunk;
  if (cthreads) *cthreads = d.cthreads;
  return EA_OK;
}

static int sp_sweeps(ea_sp *c, int n) {
  const SpGraph &g = c->g;
  for (int s = 0; s < n; ++s)
    for (int k = 0; k < g.ncol; ++k)
      SCU(sp_launch_pass(c->d, k, g.col_off[k], g.col_off[k + 1] - g.col_off[k], c->st));
  return EA_OK;
}

int ea_sp_sweeps(ea_sp *c, int32_t n) {
  if (!c || n < 0) return spfail(EA_ERR_ARG, "bad arguments");
  if (!c->have_temps) return spfail(EA_ERR_STATE, "temperatures not set");
  SCU(cudaSetDevice(c->device));
  return sp_sweeps(c, n);
}

int ea_sp_energy(ea_sp *c, int32_t *U2) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  SCU(cudaSetDevice(c->device));
  SCU(sp_launch_energy(c->d, c->st));
  if (U2) {
    SCU(cudaMemcpyAsync(U2, c->d.U2, sizeof(int32_t) * (size_t)c->d.nw * 64 * c->d.NR * c->d.NB,
                        cudaMemcpyDeviceToHost, c->st));
    SCU(cudaStreamSynchronize(c->st));
  }
  return EA_OK;
}

static int sp_pt(ea_sp *c) {
  SCU(sp_launch_energy(c->d, c->st));
  SCU(sp_launch_pt(c->d, c->st));
  SCU(sp_launch_permute(c->d, c->st));
  return EA_OK;
}

int ea_sp_parallel_tempering(ea_sp *c) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  if (!c->have_temps) return spfail(EA_ERR_STATE, "temperatures not set");
  SCU(cudaSetDevice(c->device));
  return sp_pt(c);
}

int ea_sp_get_tempering(ea_sp *c, int32_t *E, uint8_t *perm, uint32_t *acc, uint64_t *masks) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  const SpDev &d = c->d;
  const size_t n = (size_t)d.nw * 64 * d.NR * d.NB;
  SCU(cudaSetDevice(c->device));
  if (E) SCU(cudaMemcpyAsync(E, d.E, n * 4, cudaMemcpyDeviceToHost, c->st));
  if (perm) SCU(cudaMemcpyAsync(perm, d.perm, n, cudaMemcpyDeviceToHost, c->st));
  if (acc) SCU(cudaMemcpyAsync(acc, d.acc, (size_t)d.nw * 64 * d.NR * (d.NB - 1) * 4, cudaMemcpyDeviceToHost, c->st));
  if (masks) SCU(cudaMemcpyAsync(masks, d.M, (size_t)d.nw * d.NR * (d.NB - 1) * 8, cudaMemcpyDeviceToHost, c->st));
  SCU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

// Overlap buffer for moves on nclust slots (allocated before any capture).
static int sp_cluster_prepare(ea_sp *c, int &nclust) {
  SpDev &d = c->d;
  if (d.NR < 2) return spfail(EA_ERR_ARG, "the Houdayer move needs 2 replicas");
  if (nclust <= 0) nclust = (int)std::lround(0.5 * d.NB);
  if (nclust > d.NB) nclust = d.NB;
  if (nclust > c->q_cap) {
    SCU(cudaStreamSynchronize(c->st));
    if (d.Q) cudaFree(d.Q);
    if (d.cscratch) cudaFree(d.cscratch);
    if (d.slab_lab) cudaFree(d.slab_lab);
    if (d.slab_coin) cudaFree(d.slab_coin);
    d.Q = nullptr;
    d.cscratch = nullptr;
    d.slab_lab = nullptr;
    d.slab_coin = nullptr;
    d.slabD = 0;
    SCU(cudaMalloc((void **)&d.Q, sizeof(unsigned long long) * (size_t)d.nw * nclust * d.V));
    if (d.V > kSpClusterMaxV) {
      SCU(cudaMalloc((void **)&d.cscratch, sizeof(uint32_t) * sp_cluster_words(d.V) * (size_t)d.nw * nclust * 8));
      const int D = sp_slab_planes(d.L, d.Lz, d.nw, nclust);
      if (D > 0) {
        const size_t units = (size_t)d.nw * nclust * 8;
        SCU(cudaMalloc((void **)&d.slab_lab, sizeof(uint32_t) * units * 8 * d.V));
        SCU(cudaMalloc((void **)&d.slab_coin, units * d.V));
        d.slabD = D;
      }
    }
    c->q_cap = nclust;
  }
  d.nclust = nclust;
  return EA_OK;
}

static int sp_houdayer(ea_sp *c, int nclust) {
  const int rc = sp_cluster_prepare(c, nclust);
  if (rc) return rc;
  SCU(sp_launch_houdayer(c->d, c->st));
  return EA_OK;
}

int ea_sp_houdayer(ea_sp *c, int32_t nclust) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  SCU(cudaSetDevice(c->device));
  return sp_houdayer(c, nclust);
}

// EA_BIN_AUTO takes the graph.  Measured on GB300: a job alone, each phase of
// a small job is a latency-bound chain that a barrier does not shorten, and
// the graph's per-phase kernels run at twice the persistent kernel's
// occupancy (84 vs 106 us per sweep at L=6, Lz=24, NT=12); 64 small jobs of
// the serving mix, the phases in lock-step wait for each phase's slowest
// job, while the jobs' graphs on their own streams interleave (0.20 vs 0.42
// spin-updates/ps).
static bool sp_use_persist(int mode, const SpDev &) { return mode == EA_BIN_PERSISTENT; }

// The work list of the job alone (its blocks of every kind, as a batch of
// one), uploaded when the descriptor changed; then one cooperative launch.
static int sp_run_persist(ea_sp *c, const ea_cadence *cad) {
  const SpDev &d = c->d;
  if (d.ncol > kSpBatchMaxColours) return spfail(EA_ERR_ARG, "the persistent bin kernel takes up to %d colours", kSpBatchMaxColours);
  if (!c->p_jobs) {
    SCU(cudaMalloc((void **)&c->p_jobs, sizeof(SpDev)));
    SCU(cudaMalloc((void **)&c->p_pre, sizeof(uint32_t) * SPB_COUNT * 2));
    SCU(cudaMalloc((void **)&c->p_bar, sizeof(unsigned long long)));
    SCU(cudaMalloc((void **)&c->p_err, sizeof(int)));
    SCU(cudaMemsetAsync(c->p_err, 0, sizeof(int), c->st));
  }
  uint32_t cnt[SPB_COUNT];
  sp_batch_blocks(d, cad->cluster != 0, cnt);
  if (!c->p_valid || std::memcmp(&c->p_up, &d, sizeof(SpDev))) {
    std::vector<uint32_t> pre((size_t)SPB_COUNT * 2);
    for (int k = 0; k < SPB_COUNT; ++k) { pre[2 * k] = 0; pre[2 * k + 1] = cnt[k]; }
    SCU(cudaStreamSynchronize(c->st));
    SCU(cudaMemcpy(c->p_jobs, &d, sizeof(SpDev), cudaMemcpyHostToDevice));
    SCU(cudaMemcpy(c->p_pre, pre.data(), sizeof(uint32_t) * pre.size(), cudaMemcpyHostToDevice));
    c->p_up = d;
    c->p_valid = true;
  }
  SpPersistDev p{};
  p.b.jobs = c->p_jobs;
  p.b.njobs = 1;
  for (int k = 0; k < SPB_COUNT; ++k) { p.b.pre[k] = c->p_pre + 2 * k; p.b.total[k] = cnt[k]; }
  p.itmax = cad->itmax; p.houfr = cad->houfr; p.mesfr = cad->mesfr; p.ptfr = cad->ptfr;
  p.cluster = cad->cluster != 0 && d.nclust > 0;
  p.ncol_max = d.ncol;
  p.bar = c->p_bar;
  p.err = c->p_err;
  size_t smem = std::max(sp_sweep_smem(d.NB, d.NR, d.kt), (size_t)kPermRows * (d.NB | 1) * 8);
  if (p.cluster) smem = std::max(smem, sp_cluster_smem(d.V));
  const int grid = sp_persist_grid(p.b, smem);
  if (grid < 1) return spfail(EA_ERR_CUDA, "persistent bin kernel: no co-resident grid for %zu bytes of shared memory", smem);
  SCU(sp_launch_persist(p, grid, smem, c->st));
  return EA_OK;
}

static bool sp_res_ok(ea_sp *c) {
  if (c->r_state == 0 || std::memcmp(&c->r_dev, &c->d, sizeof(SpDev))) {
    c->r_state = sp_res_plan(c->d, c->g.col_sites.data(), c->expoff.empty() ? 0 : c->expoff.back(), c->r_plan) ? 1 : 2;
    c->r_dev = c->d;
  }
  return c->r_state == 1;
}

// The resident path takes bins without cluster moves of jobs that fit one
// cluster: explicitly (EA_BIN_RESIDENT) or by default.
static bool sp_use_resident(ea_sp *c, const ea_cadence *cad) {
  if (c->bin_mode != EA_BIN_RESIDENT && c->bin_mode != EA_BIN_AUTO) return false;
  return sp_res_launch_sweeps(c->d.V, (size_t)c->d.NR * c->d.NB, cad) > 0 && sp_res_ok(c);
}

static int sp_run_resident(ea_sp *c, const ea_cadence *cad) {
  const SpDev &d = c->d;
  const SpResPlan &pl = c->r_plan;
  const int spi = cad->mesfr * cad->houfr * cad->ptfr;  // sweeps per iteration
  const size_t words_sweep = (size_t)3 * d.V * d.NR * d.NB;
  const size_t nsweep = sp_res_launch_sweeps(d.V, (size_t)d.NR * d.NB, cad), npass = nsweep * d.ncol;
  const int ipl = cad->cluster ? 1 : (int)(nsweep / spi);  // iterations per launch
  const size_t npt = nsweep / cad->ptfr;                    // tempering steps per launch
  if (npass > c->r_cap_pass || nsweep > c->r_cap_sweep || npt > c->r_cap_pt) {
    SCU(cudaStreamSynchronize(c->st));
    if (c->r_ctrs) cudaFree(c->r_ctrs);
    if (c->r_R) cudaFree(c->r_R);
    if (c->r_X) cudaFree(c->r_X);
    c->r_ctrs = nullptr;
    c->r_R = c->r_X = nullptr;
    c->r_cap_pass = c->r_cap_sweep = c->r_cap_pt = 0;
    SCU(cudaMalloc((void **)&c->r_ctrs, sizeof(uint4) * npass * d.NR));
    SCU(cudaMalloc((void **)&c->r_R, 8 * words_sweep * nsweep));
    SCU(cudaMalloc((void **)&c->r_X, 8 * npt * d.nw * d.NR * (d.NB - 1) * 64));
    c->r_cap_pass = npass;
    c->r_cap_sweep = nsweep;
    c->r_cap_pt = npt;
  }
  SpResDev p{};
  p.d = d;
  p.R = c->r_R;
  p.X = c->r_X;
  p.pair_energy = c->pair_energy ? 1 : 0;
  p.houfr = cad->houfr;
  p.mesfr = cad->mesfr;
  p.ptfr = cad->ptfr;
  p.ncta = pl.ncta;
  p.nslm = pl.nslm;
  p.upc = pl.upc;
  p.ntab = pl.ntab;
  p.lpc_count = pl.lpc_count;
  p.lpc_energy = pl.lpc_energy;
  std::memcpy(p.kr, pl.kr, sizeof(p.kr));
  if (cad->cluster) {
    // per houfr block: one resident launch (sweeps and tempering steps, no
    // measurement), then the move's kernels on the words it wrote back; the
    // energies counted again and measured after each iteration, as the
    // graph path does
    p.nit = 1;
    p.mesfr = 1;
    p.nsweep = (int)nsweep;
    p.measure = 0;
    for (int it = 0; it < cad->itmax; ++it) {
      for (int im = 0; im < cad->mesfr; ++im) {
        SCU(sp_res_chunk(p, pl, p.nsweep * d.ncol, c->r_ctrs, c->st));
        SCU(sp_launch_houdayer(c->d, c->st));
      }
      SCU(sp_launch_energy(c->d, c->st));
      SCU(sp_launch_measure_u2(c->d, false, c->st));
    }
    return EA_OK;
  }
  p.measure = 1;
  for (int done = 0; done < cad->itmax;) {
    p.nit = std::min(ipl, cad->itmax - done);
    p.nsweep = p.nit * spi;
    SCU(sp_res_chunk(p, pl, p.nsweep * d.ncol, c->r_ctrs, c->st));
    done += p.nit;
  }
  return EA_OK;
}

int ea_sp_bin_kernel_for(ea_sp *c, const ea_cadence *cad, int32_t *mode) {
  if (!c || !cad || !mode || cad->itmax < 1 || cad->houfr < 1 || cad->mesfr < 1 || cad->ptfr < 1)
    return spfail(EA_ERR_ARG, "bad arguments");
  SCU(cudaSetDevice(c->device));
  if (sp_use_resident(c, cad)) *mode = EA_BIN_RESIDENT;
  else if (c->bin_mode == EA_BIN_RESIDENT) return spfail(EA_ERR_ARG, "the resident bin kernel does not take this bin");
  else *mode = c->bin_mode == EA_BIN_PERSISTENT ? EA_BIN_PERSISTENT : EA_BIN_GRAPH;
  return EA_OK;
}

int ea_sp_run(ea_sp *c, const ea_cadence *cad, double *avgE) {
  if (!c || !cad || cad->itmax < 1 || cad->houfr < 1 || cad->mesfr < 1 || cad->ptfr < 1)
    return spfail(EA_ERR_ARG, "bad cadence");
  if (!c->have_temps) return spfail(EA_ERR_STATE, "temperatures not set");
  SCU(cudaSetDevice(c->device));
  const SpDev &d = c->d;
  const size_t n = (size_t)d.nw * 64 * d.NR * d.NB;
  SCU(cudaMemsetAsync(d.avgE, 0, n * 8, c->st));
  int rc, nclust = cad->nclust;
  if (cad->cluster && (rc = sp_cluster_prepare(c, nclust))) return rc;
  if (c->bin_mode == EA_BIN_RESIDENT && !sp_use_resident(c, cad))
    return spfail(EA_ERR_ARG, "the resident bin kernel takes jobs whose words fit one thread-block cluster, bins "
                              "without cluster moves or with at least %d sweeps between moves", kResMinBlock);
  if (sp_use_resident(c, cad)) {
    if ((rc = sp_run_resident(c, cad))) return rc;
    c->last_itmax = cad->itmax;
    if (avgE) return ea_sp_bin_results(c, avgE);
    return EA_OK;
  }
  if (sp_use_persist(c->bin_mode, d)) {
    if ((rc = sp_run_persist(c, cad))) return rc;
    c->last_itmax = cad->itmax;
    if (avgE) return ea_sp_bin_results(c, avgE);
    return EA_OK;
  }
  // one iteration: every launch reads its counters (pass, tempering step,
  // move) from the device, so the captured graph replays each iteration
  auto iteration = [&]() -> int {
    for (int im = 0; im < cad->mesfr; ++im) {
      for (int ih = 0; ih < cad->houfr; ++ih) {
        int r = sp_sweeps(c, cad->ptfr);
        if (!r) r = sp_pt(c);
        if (r) return r;
      }
      if (cad->cluster) SCU(sp_launch_houdayer(c->d, c->st));
    }
    // without cluster moves the last tempering step's energies are current
    if (cad->cluster) SCU(sp_launch_energy(c->d, c->st));
    SCU(sp_launch_measure_u2(c->d, !cad->cluster, c->st));
    return EA_OK;
  };
  if (cad->itmax == 1) {
    if ((rc = iteration())) return rc;
  } else {
    if (!c->it_graph || std::memcmp(&c->it_cad, cad, sizeof(ea_cadence)) ||
        std::memcmp(&c->it_dev, &c->d, sizeof(SpDev))) {
      if (c->it_graph) { cudaGraphExecDestroy(c->it_graph); c->it_graph = nullptr; }
      cudaGraph_t graph = nullptr;
      SCU(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
      rc = iteration();
      const cudaError_t e = cudaStreamEndCapture(c->st, &graph);
      if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
      SCU(e);
      const cudaError_t ei = cudaGraphInstantiate(&c->it_graph, graph, 0);
      cudaGraphDestroy(graph);
      SCU(ei);
      c->it_cad = *cad;
      c->it_dev = c->d;
    }
    for (int it = 0; it < cad->itmax; ++it) SCU(cudaGraphLaunch(c->it_graph, c->st));
  }
  c->last_itmax = cad->itmax;
  if (avgE) return ea_sp_bin_results(c, avgE);
  return EA_OK;
}

int ea_sp_bin_results(ea_sp *c, double *avgE) {
  if (!c || !avgE) return spfail(EA_ERR_ARG, "null argument");
  if (c->last_itmax < 1) return spfail(EA_ERR_STATE, "no bin has run");
  SCU(cudaSetDevice(c->device));
  const SpDev &d = c->d;
  const size_t n = (size_t)d.nw * 64 * d.NR * d.NB;
  std::vector<double> h(n);
  SCU(cudaMemcpyAsync(h.data(), d.avgE, n * 8, cudaMemcpyDeviceToHost, c->st));
  SCU(cudaStreamSynchronize(c->st));
  const int rc = sp_check_persist(c->p_err, c->st);
  if (rc) return rc;
  for (size_t i = 0; i < n; ++i) avgE[i] = h[i] / c->last_itmax;
  return EA_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches of sample-packed jobs
// ---------------------------------------------------------------------------
// A batch is split into classes -- one per job for batches of up to
// kSpBatchBranches jobs, else jobs with the same number of temperatures and
// lattices of similar size -- so that every launch is sized for its class
// (SMEM of the thresholds and of the cluster labelling, labelling block
// size); each class's bin iteration is a branch of one CUDA graph, so the
// classes run side by side and one graph launch advances the whole batch.
// (Measured on 72 jobs of mixed geometry: one class per job 0.83x / 0.97x of
// the jobs on their own streams for 72 / 1024 sample words, (NB, size)
// classes 0.78x / 0.90x, a single class 0.62x / 0.70x: fusing different
// geometries into one launch costs more than the launches it saves.)
struct SpClass {
  std::vector<ea_sp *> jobs;
  int ncol_max = 0, cl_threads = 1024;
  SpDev *d_jobs = nullptr;
  uint32_t *d_pre = nullptr;
  std::vector<SpDev> up_jobs;
  std::vector<uint32_t> up_pre;
  SpBatchDev bd{};
  cudaStream_t fs = nullptr;   // branch stream of the capture
  cudaEvent_t join = nullptr;
};

struct ea_sp_batch {
  std::vector<SpClass> classes;
  std::vector<ea_sp *> jobs;
  int device = 0;
  cudaStream_t bs = nullptr;
  cudaEvent_t done = nullptr, fork = nullptr;
  cudaGraphExec_t it_graph = nullptr;
  ea_cadence it_cad{};
  std::vector<SpBatchDev> it_bd;
  // persistent bin kernel: every job in one work list
  int bin_mode = EA_BIN_AUTO;
  SpClass all;
  unsigned long long *p_bar = nullptr;
  int *p_err = nullptr;
};

constexpr int kSpBatchBranches = 256;

static int sp_size_bucket(int V) { return V <= 2048 ? 0 : V <= 8192 ? 1 : V <= kSpClusterMaxV ? 2 : 3; }

static int spb_upload(SpClass &k, bool cluster, cudaStream_t bs) {
  const int n = (int)k.jobs.size();
  std::vector<SpDev> hj(n);
  std::vector<uint32_t> hp((size_t)SPB_COUNT * (n + 1), 0);
  int pass_smem = 0, perm_smem = 0, cl_smem = 0;
  for (int i = 0; i < n; ++i) {
    hj[i] = k.jobs[i]->d;
    uint32_t cnt[SPB_COUNT];
    sp_batch_blocks(hj[i], cluster, cnt);
    for (int q = 0; q < SPB_COUNT; ++q) hp[(size_t)q * (n + 1) + i + 1] = hp[(size_t)q * (n + 1) + i] + cnt[q];
    pass_smem = std::max(pass_smem, (int)(hj[i].pgrid ? sp_items_smem(hj[i].NB)
                                                       : sp_sweep_smem(hj[i].NB, hj[i].NR, hj[i].kt)));
    perm_smem = std::max(perm_smem, kPermRows * (hj[i].NB | 1) * 8);
    if (cluster) cl_smem = std::max(cl_smem, (int)sp_cluster_smem(hj[i].V));
  }
  if (k.up_jobs.size() != hj.size() || std::memcmp(k.up_jobs.data(), hj.data(), sizeof(SpDev) * n) ||
      k.up_pre != hp) {
    SCU(cudaStreamSynchronize(bs));
    SCU(cudaMemcpy(k.d_jobs, hj.data(), sizeof(SpDev) * n, cudaMemcpyHostToDevice));
    SCU(cudaMemcpy(k.d_pre, hp.data(), sizeof(uint32_t) * hp.size(), cudaMemcpyHostToDevice));
    k.up_jobs = hj;
    k.up_pre = hp;
  }
  SpBatchDev &bd = k.bd;
  bd = SpBatchDev{};
  bd.jobs = k.d_jobs;
  bd.njobs = n;
  for (int q = 0; q < SPB_COUNT; ++q) {
    bd.pre[q] = k.d_pre + (size_t)q * (n + 1);
    bd.total[q] = hp[(size_t)q * (n + 1) + n];
  }
  bd.pass_smem = pass_smem;
  bd.perm_smem = perm_smem;
  bd.cluster_smem = cl_smem;
  bd.cluster_threads = k.cl_threads;
  return EA_OK;
}

static cudaError_t spb_iteration(const SpClass &k, const ea_cadence *cad, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  for (int im = 0; im < cad->mesfr && e == cudaSuccess; ++im) {
    for (int ih = 0; ih < cad->houfr && e == cudaSuccess; ++ih) {
      for (int sw = 0; sw < cad->ptfr && e == cudaSuccess; ++sw) e = sp_batch_sweep(k.bd, k.ncol_max, st);
      if (e == cudaSuccess) e = sp_batch_tempering(k.bd, st);
    }
    if (e == cudaSuccess && cad->cluster) e = sp_batch_houdayer(k.bd, st);
  }
  if (e == cudaSuccess) e = sp_batch_measure(k.bd, !cad->cluster, st);
  return e;
}

extern "C" {

int ea_sp_batch_create(ea_sp *const *jobs, int32_t njobs, ea_sp_batch **out) {
  if (!jobs || !out || njobs < 1) return spfail(EA_ERR_ARG, "at least one job");
  ea_sp_batch *b = new ea_sp_batch();
  std::vector<std::pair<int, int>> keys;
  for (int i = 0; i < njobs; ++i) {
    ea_sp *c = jobs[i];
    if (!c || std::find(b->jobs.begin(), b->jobs.end(), c) != b->jobs.end()) {
      delete b;
      return spfail(EA_ERR_ARG, "job %d is null or appears twice", i);
    }
    if (i && c->device != b->device) { delete b; return spfail(EA_ERR_ARG, "the jobs of a batch share the device"); }
    if (c->d.ncol > kSpBatchMaxColours) {
      delete b;
      return spfail(EA_ERR_ARG, "job %d needs %d colours (a batch takes %d)", i, c->d.ncol, kSpBatchMaxColours);
    }
    b->device = c->device;
    b->jobs.push_back(c);
    // one class per job up to kSpBatchBranches jobs (measured fastest: every
    // launch sized for its job, the jobs' branches side by side), else
    // classes of equal NB and lattice-size bucket
    const std::pair<int, int> key(njobs <= kSpBatchBranches ? i : c->d.NB, sp_size_bucket(c->d.V));
    size_t q = std::find(keys.begin(), keys.end(), key) - keys.begin();
    if (q == keys.size()) {
      keys.push_back(key);
      b->classes.emplace_back();
      b->classes.back().cl_threads = sp_cluster_threads(key.second == 0 ? 2048 : 32768);
    }
    SpClass &k = b->classes[q];
    k.jobs.push_back(c);
    k.ncol_max = std::max(k.ncol_max, c->d.ncol);
  }
  cudaError_t e = cudaSetDevice(b->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->bs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  b->all.jobs = b->jobs;
  for (ea_sp *c : b->jobs) b->all.ncol_max = std::max(b->all.ncol_max, c->d.ncol);
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->all.d_jobs, sizeof(SpDev) * b->jobs.size());
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->all.d_pre, sizeof(uint32_t) * SPB_COUNT * (b->jobs.size() + 1));
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->p_bar, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc((void **)&b->p_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(b->p_err, 0, sizeof(int));
  for (SpClass &k : b->classes) {
    const size_t n = k.jobs.size();
    if (e == cudaSuccess) e = cudaMalloc((void **)&k.d_jobs, sizeof(SpDev) * n);
    if (e == cudaSuccess) e = cudaMalloc((void **)&k.d_pre, sizeof(uint32_t) * SPB_COUNT * (n + 1));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&k.fs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&k.join, cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = sp_batch_setup();
  if (e != cudaSuccess) {
    ea_sp_batch_destroy(b);
    return spfail(EA_ERR_CUDA, "batch set-up: %s", cudaGetErrorString(e));
  }
  *out = b;
  return EA_OK;
}

int ea_sp_batch_destroy(ea_sp_batch *b) {
  if (!b) return EA_OK;
  cudaSetDevice(b->device);
  if (b->bs) cudaStreamSynchronize(b->bs);
  if (b->it_graph) cudaGraphExecDestroy(b->it_graph);
  for (SpClass &k : b->classes) {
    if (k.d_jobs) cudaFree(k.d_jobs);
    if (k.d_pre) cudaFree(k.d_pre);
    if (k.join) cudaEventDestroy(k.join);
    if (k.fs) cudaStreamDestroy(k.fs);
  }
  if (b->all.d_jobs) cudaFree(b->all.d_jobs);
  if (b->all.d_pre) cudaFree(b->all.d_pre);
  if (b->p_bar) cudaFree(b->p_bar);
  if (b->p_err) cudaFree(b->p_err);
  if (b->done) cudaEventDestroy(b->done);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->bs) cudaStreamDestroy(b->bs);
  delete b;
  return EA_OK;
}

int ea_sp_batch_stream(ea_sp_batch *b, void **stream) {
  if (!b || !stream) return spfail(EA_ERR_ARG, "null argument");
  *stream = (void *)b->bs;
  return EA_OK;
}

int ea_sp_batch_sync(ea_sp_batch *b) {
  if (!b) return spfail(EA_ERR_ARG, "null batch");
  SCU(cudaSetDevice(b->device));
  SCU(cudaStreamSynchronize(b->bs));
  return sp_check_persist(b->p_err, b->bs);
}

int ea_sp_batch_set_bin_kernel(ea_sp_batch *b, int32_t mode) {
  if (!b || mode < EA_BIN_AUTO || mode > EA_BIN_PERSISTENT) return spfail(EA_ERR_ARG, "bad bin-kernel mode");
  b->bin_mode = mode;
  return EA_OK;
}

int ea_sp_batch_run(ea_sp_batch *b, const ea_cadence *cad) {
  if (!b || !cad || cad->itmax < 1 || cad->houfr < 1 || cad->mesfr < 1 || cad->ptfr < 1)
    return spfail(EA_ERR_ARG, "bad cadence");
  SCU(cudaSetDevice(b->device));
  int rc;
  for (ea_sp *c : b->jobs) {
    if (!c->have_temps) return spfail(EA_ERR_STATE, "temperatures not set");
    int nclust = cad->nclust;
    if (cad->cluster && (rc = sp_cluster_prepare(c, nclust))) return rc;
    // every job's earlier work comes first
    SCU(cudaEventRecord(b->done, c->st));
    SCU(cudaStreamWaitEvent(b->bs, b->done, 0));
  }
  const bool persist = b->bin_mode == EA_BIN_PERSISTENT;
  if (persist) {
    // one work list of every job, one cooperative launch per bin
    if ((rc = spb_upload(b->all, cad->cluster != 0, b->bs))) return rc;
    for (ea_sp *c : b->jobs)
      SCU(cudaMemsetAsync(c->d.avgE, 0, sizeof(double) * (size_t)c->d.nw * 64 * c->d.NR * c->d.NB, b->bs));
    SpPersistDev p{};
    p.b = b->all.bd;
    p.itmax = cad->itmax; p.houfr = cad->houfr; p.mesfr = cad->mesfr; p.ptfr = cad->ptfr;
    p.cluster = cad->cluster != 0;
    p.ncol_max = b->all.ncol_max;
    p.bar = b->p_bar;
    p.err = b->p_err;
    const size_t smem = (size_t)std::max(std::max(p.b.pass_smem, p.b.perm_smem), p.b.cluster_smem);
    const int grid = sp_persist_grid(p.b, smem);
    if (grid < 1) return spfail(EA_ERR_CUDA, "persistent bin kernel: no co-resident grid for %zu bytes of shared memory", smem);
    SCU(sp_launch_persist(p, grid, smem, b->bs));
  } else {
  std::vector<SpBatchDev> bds;
  for (SpClass &k : b->classes) {
    if ((rc = spb_upload(k, cad->cluster != 0, b->bs))) return rc;
    bds.push_back(k.bd);
  }
  for (ea_sp *c : b->jobs)
    SCU(cudaMemsetAsync(c->d.avgE, 0, sizeof(double) * (size_t)c->d.nw * 64 * c->d.NR * c->d.NB, b->bs));
  if (!b->it_graph || std::memcmp(&b->it_cad, cad, sizeof(ea_cadence)) || b->it_bd.size() != bds.size() ||
      std::memcmp(b->it_bd.data(), bds.data(), sizeof(SpBatchDev) * bds.size())) {
    if (b->it_graph) { cudaGraphExecDestroy(b->it_graph); b->it_graph = nullptr; }
    cudaGraph_t graph = nullptr;
    SCU(cudaStreamBeginCapture(b->bs, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaEventRecord(b->fork, b->bs);
    for (SpClass &k : b->classes) {
      if (e == cudaSuccess) e = cudaStreamWaitEvent(k.fs, b->fork, 0);
      if (e == cudaSuccess) e = spb_iteration(k, cad, k.fs);
      if (e == cudaSuccess) e = cudaEventRecord(k.join, k.fs);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(b->bs, k.join, 0);
    }
    const cudaError_t ec = cudaStreamEndCapture(b->bs, &graph);
    if (e != cudaSuccess || ec != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return spfail(EA_ERR_CUDA, "batch capture: %s", cudaGetErrorString(e != cudaSuccess ? e : ec));
    }
    const cudaError_t ei = cudaGraphInstantiate(&b->it_graph, graph, 0);
    cudaGraphDestroy(graph);
    SCU(ei);
    b->it_cad = *cad;
    b->it_bd = bds;
  }
  for (int it = 0; it < cad->itmax; ++it) SCU(cudaGraphLaunch(b->it_graph, b->bs));
  }
  // later work of each job comes after the batch
  SCU(cudaEventRecord(b->done, b->bs));
  for (ea_sp *c : b->jobs) {
    SCU(cudaStreamWaitEvent(c->st, b->done, 0));
    c->last_itmax = cad->itmax;
  }
  return EA_OK;
}

int ea_sp_job_bytes(const ea_sp_geom *gp, const ea_cadence *cad, const double *betas, uint64_t *bytes) {
  SpGraph g;
  if (!bytes || !geom_ok(gp) || !sp_graph(gp->L, gp->Lz, gp->bc, g)) return spfail(EA_ERR_ARG, "bad sample-packed geometry");
  uint64_t tot = 0;
  auto add = [&](uint64_t n) {
    n = std::max<uint64_t>(n, 1);
    tot += n >= (1ull << 20) ? (n + (2ull << 20) - 1) & ~((2ull << 20) - 1) : (n + 511) & ~(uint64_t)511;
  };
  const uint64_t V = g.V, NB = gp->nbetas, NR = gp->nrep, nw = gp->nwords, G = NR * NB;
  add(V * 24); add(V * 4);                                   // neighbour table, colour lists
  add(nw * V * G * 8); add(nw * V * 48);                     // spins, couplings
  add(NB * 256 * 8); add(NB * 256 * 2); add(NB * kPre11Stride);  // thresholds, pre-searches
  add(NR * 16); add(NR * 4); add(NR * sizeof(ea_hq)); add(NR * sizeof(ea_xoshiro)); add(8);
  add(nw * 64 * G * 4); add(nw * 64 * G * 4); add(nw * 64 * G);   // U2, E, slot permutations
  add(nw * 64 * NR * (NB - 1) * 4); add(nw * NR * (NB - 1) * 8); // accepted swaps, lane masks
  add(NB * 8); add(NB * 4); add(8); add(nw * 64 * G * 8);   // betas, exp offsets, step, averages
  add(sizeof(ea_hq)); add(16); add(8);                      // random_c, pairs, move counter
  uint64_t nexp = (NB - 1) * 25001;
  if (betas) {
    std::vector<double> tab;
    std::vector<int32_t> off;
    pt_exp_table(betas, (int)NB, tab, off);
    nexp = tab.size();
  }
  add(nexp * 8);
  if (cad && cad->cluster) {
    const uint64_t nc = (uint64_t)(cad->nclust > 0 ? std::min<int>(cad->nclust, (int)NB) : std::lround(0.5 * NB));
    add(nw * nc * V * 8);
    if (V > (uint64_t)kSpClusterMaxV) add(nw * nc * 8 * sp_cluster_words((int)V) * 4);
    if (sp_slab_planes(gp->L, gp->Lz, (int)nw, (int)nc) > 0) {   // slab labels and coins
      add(nw * nc * 8 * 8 * V * 4);
      add(nw * nc * 8 * V);
    }
  }
  if (cad && sp_res_fits(gp->L, gp->Lz, (int)nw, (int)NR, (int)NB)) {
    // the resident kernel's counters, random words and tempering uniforms
    const uint64_t ns = sp_res_launch_sweeps(V, G, cad);
    add(ns * g.ncol * NR * 16);
    add(ns * 24 * V * G);
    if (cad->ptfr > 0) add(ns / cad->ptfr * nw * NR * (NB - 1) * 64 * 8);
  }
  *bytes = tot + (2ull << 20);                               // stream, graph, small-allocation pages
  return EA_OK;
}

int ea_sp_exact(ea_sp *c, const double *betas, int32_t nbeta, uint64_t *dos, double *meanE) {
  if (!c) return spfail(EA_ERR_ARG, "null job");
  const SpDev &d0 = c->d;
  if (d0.V > 32) return spfail(EA_ERR_ARG, "exact enumeration needs V <= 32 sites (V = %d)", d0.V);
  if (meanE && (!betas || nbeta < 1)) return spfail(EA_ERR_ARG, "betas");
  SCU(cudaSetDevice(c->device));
  const size_t nbins = 6 * (size_t)d0.V + 1, ns = (size_t)d0.nw * 64;
  if (!c->d.dos) SCU(cudaMalloc((void **)&c->d.dos, ns * nbins * 8));
  const SpDev &d = c->d;
  SCU(cudaMemsetAsync(d.dos, 0, ns * nbins * 8, c->st));
  SCU(sp_launch_dos(d, c->st));
  if (dos) SCU(cudaMemcpyAsync(dos, d.dos, ns * nbins * 8, cudaMemcpyDeviceToHost, c->st));
  if (meanE) {
    double *db = nullptr, *dm = nullptr;
    SCU(cudaMalloc((void **)&db, sizeof(double) * nbeta));
    SCU(cudaMalloc((void **)&dm, sizeof(double) * ns * nbeta));
    SCU(cudaMemcpyAsync(db, betas, sizeof(double) * nbeta, cudaMemcpyHostToDevice, c->st));
    SCU(sp_launch_exact(d, db, nbeta, dm, c->st));
    SCU(cudaMemcpyAsync(meanE, dm, sizeof(double) * ns * nbeta, cudaMemcpyDeviceToHost, c->st));
    SCU(cudaStreamSynchronize(c->st));
    cudaFree(db);
    cudaFree(dm);
  }
  SCU(cudaStreamSynchronize(c->st));
  return EA_OK;
}

}  // extern "C"
