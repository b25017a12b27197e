/*
 * sp_oracle.c -- TEST INFRASTRUCTURE ONLY.  CPU restatement of the
 * sample-packed layout's dynamics (64 samples per word, any L, Lz), used by
 * tests/ as the checker of the CUDA kernels; nothing in the product links or
 * calls it.
 *
 * The layout has no counterpart in the reference (its words hold 64 spatial
 * sub-blocks of one sample, PROGRAM/include/header.h:41-47), so there is
 * nothing of the reference to pin it to directly.  What it restates per
 * sample is the reference's arithmetic: the random words of
 * d_gen_rndbits_cuda (main.cu:994-1150, or_rnd_triple in ea_oracle.c), the
 * bit-sliced Metropolis rule of d_oneMCstepBN_multisample
 * (main.cu:1474-1506), E = 3V - 2 x unsatisfied bonds (main.cu:1379) and the
 * tempering rule of Parallel_Tempering (upd.c:3-48).  The bond graph (which
 * site sits in which slot, the colouring) is an input: the tests take it from
 * the library's host code and check its properties separately.  The density
 * of states gives the statistical check: exact <E>(beta) against Monte Carlo.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ea_oracle.h"

/* Bit-sliced flip mask, main.cu:1474-1506: f[d] = 1 marks an unsatisfied
 * slot; b0..b2 are the three random words of the site. */
static uint64_t sp_flip(const uint64_t f[6], uint64_t b0, uint64_t b1, uint64_t b2) {
  uint64_t k1 = f[0] ^ f[1], k2 = f[0] & f[1];
  uint64_t j1 = k1 ^ f[2], j2 = k2 ^ (k1 & f[2]);
  k1 = f[3] ^ f[4]; k2 = f[3] & f[4];
  uint64_t j3 = k1 ^ f[5], j4 = k2 ^ (k1 & f[5]);
  b1 = b0 & b1; b2 = b1 & b2;
  uint64_t id2 = b1, id1 = (b0 ^ b1) | b2, j24 = j2 | j4;
  return (j1 & j3 & id1) | ((j24 | id2) & (j1 | j3 | id1)) | ((j2 & j4) | (j24 & id2));
}

/* One colour pass: sites[0..nsites) of one colour, counters ctr [NR][4] of
 * the pass.  Random words of (slot b, site i, replica r): Philox thread index
 * (b*V + i)*NR + r with the temperature's thresholds cum[b]. */
void or_sp_pass(int V, int NR, int NB, int nw, const int32_t *nb, const int32_t *sites, int nsites,
                const uint32_t *ctr, const uint32_t *keys, const uint64_t *cum, const uint64_t *J, uint64_t *S) {
  const size_t G = (size_t)NR * NB;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nsites; k++) {
    const int i = sites[k];
    for (int b = 0; b < NB; b++)
      for (int r = 0; r < NR; r++) {
        uint64_t rnd[3];
        const uint32_t tp = (uint32_t)(((size_t)b * V + i) * NR + r);
        or_rnd_triple(ctr + 4 * r, keys[r], tp, cum + (size_t)b * 256, rnd);
        for (int w = 0; w < nw; w++) {
          uint64_t *Sw = S + (size_t)w * V * G;
          const uint64_t *Jw = J + ((size_t)w * V + i) * 6;
          const size_t o = (size_t)r * NB + b;
          const uint64_t s = Sw[(size_t)i * G + o];
          uint64_t f[6];
          for (int d = 0; d < 6; d++) f[d] = s ^ Jw[d] ^ Sw[(size_t)nb[i * 6 + d] * G + o];
          Sw[(size_t)i * G + o] = s ^ sp_flip(f, rnd[0], rnd[1], rnd[2]);
        }
      }
  }
}

/* Unsatisfied half-edges per (word, sample, replica, slot): U2 [nw][64][NR][NB].
 * Per-sample counts of the unsatisfied slots f of every site: each byte of f
 * adds the 0/1 counts of its 8 samples to one 64-bit accumulator (8 bytes,
 * one per sample) through a table, flushed into int32 counters before a
 * byte can overflow. */
void or_sp_energy(int V, int NR, int NB, int nw, const int32_t *nb, const uint64_t *J, const uint64_t *S,
                  int32_t *U2) {
  const size_t G = (size_t)NR * NB;
  static uint64_t spread[256];
  static int spread_done = 0;
  if (!spread_done) {
    for (int x = 0; x < 256; x++) {
      uint64_t v = 0;
      for (int b = 0; b < 8; b++) v |= (uint64_t)((x >> b) & 1) << (8 * b);
      spread[x] = v;
    }
    spread_done = 1;
  }
  memset(U2, 0, sizeof(int32_t) * (size_t)nw * 64 * G);
#pragma omp parallel for schedule(static)
  for (int wo = 0; wo < nw * (int)G; wo++) {
    const int w = wo / (int)G, o = wo % (int)G;
    const uint64_t *Sw = S + (size_t)w * V * G;
    const uint64_t *Jw = J + (size_t)w * V * 6;
    int32_t cnt[64];
    uint64_t acc[8];
    memset(cnt, 0, sizeof(cnt));
    memset(acc, 0, sizeof(acc));
    int pending = 0;
    for (int i = 0; i < V; i++) {
      for (int d = 0; d < 6; d++) {
        const uint64_t f = Sw[(size_t)i * G + o] ^ Jw[(size_t)i * 6 + d] ^ Sw[(size_t)nb[i * 6 + d] * G + o];
        for (int k = 0; k < 8; k++) acc[k] += spread[(f >> (8 * k)) & 255];
      }
      pending += 6;
      if (pending > 240 || i == V - 1) {
        for (int k = 0; k < 8; k++) {
          for (int b = 0; b < 8; b++) cnt[8 * k + b] += (int32_t)((acc[k] >> (8 * b)) & 255);
          acc[k] = 0;
        }
        pending = 0;
      }
    }
    for (int lane = 0; lane < 64; lane++) U2[((size_t)w * 64 + lane) * G + o] = cnt[lane];
  }
}

static void philox_pt(uint32_t v[4], uint32_t k0, uint32_t k1) {
  for (int i = 0; i < 10; i++) {
    if (i) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    const uint64_t p0 = (uint64_t)0xD2511F53u * v[0], p1 = (uint64_t)0xCD9E8D57u * v[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ v[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ v[3] ^ k1;
    v[1] = (uint32_t)p1; v[3] = (uint32_t)p0; v[0] = n0; v[2] = n2;
  }
}

/* One tempering step of every (word, sample, replica) chain, upd.c:3-48:
 * pairs i = 0..NB-2 in order, dE = E[i+1] - E[i], pt = -(b[i+1]-b[i]) dE,
 * accept if pt >= 0 or FNORM*u < exp(pt).  exptab/expoff: the host-libm
 * table of exp(pt) for dE = -2m (m = 1..), beyond it only u = 0 accepts.
 * u = Philox4x32-10(step, pair, chain) keyed by the tempering seed.
 * E, perm [nw][64][NR][NB] are updated in place (swapped with the
 * configurations); masks [nw][NR][NB-1] receive the accepted lanes; then
 * the spins S move between slots. */
void or_sp_pt(int V, int NR, int NB, int nw, const double *betas, const double *exptab, const int32_t *expoff,
              uint64_t step, uint64_t seed, const int32_t *U2, int32_t *E, uint8_t *perm, uint32_t *acc,
              uint64_t *masks, uint64_t *S) {
  const size_t G = (size_t)NR * NB;
  const double FNORM = 5.4210108624275218e-20;
  memset(masks, 0, sizeof(uint64_t) * (size_t)nw * NR * (NB - 1));
  for (int w = 0; w < nw; w++)
    for (int lane = 0; lane < 64; lane++)
      for (int r = 0; r < NR; r++) {
        const size_t o = ((size_t)w * 64 + lane) * G + (size_t)r * NB;
        int32_t *e = E + o;
        uint8_t *pm = perm + o;
        for (int b = 0; b < NB; b++) e[b] = 3 * V - U2[o + b];
        const uint32_t chain = (uint32_t)(((size_t)w * 64 + lane) * NR + r);
        for (int i = 0; i < NB - 1; i++) {
          const int dE = e[i + 1] - e[i];
          const double pt = -(betas[i + 1] - betas[i]) * (double)dE;
          uint32_t v[4] = {(uint32_t)step, (uint32_t)(step >> 32), (uint32_t)i, chain};
          philox_pt(v, (uint32_t)seed, (uint32_t)(seed >> 32));
          const uint64_t u = ((uint64_t)v[0] << 32) | v[1];
          int change;
          if (pt >= 0.0) {
            change = 1;
          } else {
            const int m = (-dE) >> 1, base = expoff[i], nx = expoff[i + 1] - base;
            change = (m >= 1 && m <= nx) ? (FNORM * (double)u < exptab[base + m - 1]) : (u == 0);
          }
          if (change) {
            int32_t t = e[i]; e[i] = e[i + 1]; e[i + 1] = t;
            uint8_t q = pm[i]; pm[i] = pm[i + 1]; pm[i + 1] = q;
            acc[(((size_t)w * 64 + lane) * NR + r) * (NB - 1) + i] += 1u;
            masks[((size_t)w * NR + r) * (NB - 1) + i] |= 1ULL << lane;
          }
        }
      }
  /* configurations follow their swaps, pair by pair */
  for (int w = 0; w < nw; w++)
    for (int i = 0; i < V; i++)
      for (int r = 0; r < NR; r++) {
        uint64_t *p = S + (((size_t)w * V + i) * NR + r) * NB;
        const uint64_t *m = masks + ((size_t)w * NR + r) * (NB - 1);
        for (int k = 0; k < NB - 1; k++) {
          const uint64_t x = (p[k] ^ p[k + 1]) & m[k];
          p[k] ^= x;
          p[k + 1] ^= x;
        }
      }
}

/* Density of states of one sample (lane of word w): configurations with
 * spin 0 up at each E = 3V - U2 (hist [6V+1], E + 3V as the index), by
 * plain enumeration of all 2^(V-1) configurations in binary order.  V <= 32. */
void or_sp_dos(int V, const int32_t *nb, const uint64_t *J, int w, int lane, uint64_t *hist) {
  const int nbins = 6 * V + 1;
  memset(hist, 0, sizeof(uint64_t) * nbins);
  uint8_t j[32 * 6];
  for (int h = 0; h < 6 * V; h++) j[h] = (uint8_t)((J[(size_t)w * V * 6 + h] >> lane) & 1ULL);
  const uint64_t n = 1ULL << (V - 1);
#pragma omp parallel
  {
    uint64_t *loc = (uint64_t *)calloc(nbins, sizeof(uint64_t));
#pragma omp for schedule(static)
    for (int64_t c = 0; c < (int64_t)n; c++) {
      const uint64_t s = (uint64_t)c << 1;
      int U2 = 0;
      for (int i = 0; i < V; i++) {
        const int si = (int)((s >> i) & 1ULL);
        for (int d = 0; d < 6; d++) U2 += si ^ (int)((s >> nb[i * 6 + d]) & 1ULL) ^ j[i * 6 + d];
      }
      loc[6 * V - U2]++;
    }
#pragma omp critical
    for (int b = 0; b < nbins; b++) hist[b] += loc[b];
    free(loc);
  }
}

/* One group of a Houdayer move on the slots b < nclust of every sample:
 * q = s_r1 ^ s_r2, maximal clusters of equal q along the six bond slots,
 * each labelled by its smallest site (a depth-first walk started from the
 * sites in ascending order), flipped in both replicas when the lowest bit of
 * Philox4x32-10((move, root, tag), key) is 1, tag = ((w*64 + lane) << 6 | b) << 1 | g. */
void or_sp_cluster(int V, int NR, int NB, int nw, const int32_t *nb, int nclust, int g, int r1, int r2,
                   uint64_t move, uint64_t key, uint64_t *S) {
  const size_t G = (size_t)NR * NB;
#pragma omp parallel
  {
    int32_t *root = (int32_t *)malloc(sizeof(int32_t) * V);
    int32_t *stack = (int32_t *)malloc(sizeof(int32_t) * V);
    uint8_t *q = (uint8_t *)malloc(V);
#pragma omp for schedule(dynamic) collapse(3)
    for (int w = 0; w < nw; w++)
      for (int b = 0; b < nclust; b++)
        for (int lane = 0; lane < 64; lane++) {
          uint64_t *Sw = S + (size_t)w * V * G;
          for (int i = 0; i < V; i++) {
            const uint64_t x = Sw[(size_t)i * G + (size_t)r1 * NB + b] ^ Sw[(size_t)i * G + (size_t)r2 * NB + b];
            q[i] = (uint8_t)((x >> lane) & 1ULL);
            root[i] = -1;
          }
          for (int i = 0; i < V; i++) {
            if (root[i] >= 0) continue;
            int top = 0;
            stack[top++] = i;
            root[i] = i;
            while (top) {
              const int k = stack[--top];
              for (int d = 0; d < 6; d++) {
                const int p = nb[k * 6 + d];
                if (root[p] < 0 && q[p] == q[i]) { root[p] = i; stack[top++] = p; }
              }
            }
          }
          const uint32_t tag = (((uint32_t)(w * 64 + lane) << 6 | (uint32_t)b) << 1) | (uint32_t)g;
          /* the coin of each cluster, drawn at its root (q[] is free now) */
          for (int i = 0; i < V; i++) {
            if (root[i] != i) continue;
            uint32_t v[4] = {(uint32_t)move, (uint32_t)(move >> 32), (uint32_t)i, tag};
            philox_pt(v, (uint32_t)key, (uint32_t)(key >> 32));
            q[i] = (uint8_t)(v[0] & 1u);
          }
          for (int i = 0; i < V; i++) {
            if (q[root[i]]) {
              const uint64_t bit = 1ULL << lane;
#pragma omp atomic
              Sw[(size_t)i * G + (size_t)r1 * NB + b] ^= bit;
#pragma omp atomic
              Sw[(size_t)i * G + (size_t)r2 * NB + b] ^= bit;
            }
          }
        }
    free(root);
    free(stack);
    free(q);
  }
}
