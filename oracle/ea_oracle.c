/*
 * ea_oracle.c -- CPU restatement of the EA-LCD-MC hot path (TEST INFRASTRUCTURE).
 *
 * This file is the oracle: tests compare the CUDA library against it, and the
 * reference leg of bench.py times it on host cores.  Nothing in the product
 * links it.  Each function cites the reference code it restates (paths relative
 * to the reference project, PROGRAM/...).  The restatement is pinned by the
 * fixtures in tests/golden/.
 */
#include "ea_oracle.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#ifdef OR_HAVE_CURAND
#include <curand.h>
#endif
#ifdef OR_HAVE_QUADMATH
#include <quadmath.h>
#endif

#define LCG_A 3202034522624059733ULL

/* ------------------------------------------------------------------------- */
/* Geometry (PROGRAM/include/header.h:50-66)                                  */
/* ------------------------------------------------------------------------- */
int or_geom_init(or_geom *g, int L, int Lz, int NB, int NR, int nbits, int bc) {
  if (L <= 0 || Lz <= 0 || (L % 8) || (Lz % 8)) return -1; /* header.h:41-47 */
  g->L = L; g->Lz = Lz; g->NB = NB; g->NR = NR; g->nbits = nbits; g->bc = bc;
  g->msc_l = L >> 2; g->msc_lz = Lz >> 2;
  g->msc_s = g->msc_l * g->msc_l;
  g->msc_v = g->msc_s * g->msc_lz;
  g->half = g->msc_v >> 1;
  g->V = L * L * Lz;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Host generators                                                            */
/* ------------------------------------------------------------------------- */
/* _actualiza_aleatorio_HQ_escalar, PROGRAM/include/random_generator.h:62-67 */
uint64_t or_hq_next(or_hq *u) {
  u->ira[u->ip] = u->ira[u->ip1] + u->ira[u->ip2];
  u->PR = u->ira[u->ip] ^ u->ira[u->ip3];
  u->zseed = u->zseed * LCG_A + 1;
  u->final = u->zseed + u->PR;
  u->ip++; u->ip1++; u->ip2++; u->ip3++;
  return u->final;
}

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* _actualiza_xoshiro256pp, PROGRAM/include/random_generator.h:50-59 */
uint64_t or_xo_next(or_xo *u) {
  u->final = rotl64(u->s[0] + u->s[3], 23) + u->s[0];
  u->t = u->s[1] << 17;
  u->s[2] ^= u->s[0];
  u->s[3] ^= u->s[1];
  u->s[1] ^= u->s[2];
  u->s[0] ^= u->s[3];
  u->s[2] ^= u->t;
  u->s[3] = rotl64(u->s[3], 45);
  return u->final;
}

/* Init_Rand_HQ_64bits, PROGRAM/src/random_generator.cu:160-201 */
void or_hq_init(or_hq *u, uint64_t seed) {
  or_hq s;
  memset(&s, 0, sizeof(s));
  s.zseed = seed;
  for (int i = 0; i < 111; i++) s.zseed = s.zseed * LCG_A + 1;
  for (int k = 128 - 61; k < 128; k++) {
    s.ira[k] = 0;
    for (int i = 0; i < 8; i++) {
      s.zseed = s.zseed * LCG_A + 1;
      s.ira[k] |= (s.zseed >> 56) << (8 * i);
    }
  }
  s.ip = 128; s.ip1 = 128 - 24; s.ip2 = 128 - 55; s.ip3 = 128 - 61;
  for (int i = 0; i < 1111; i++) {
    s.ira[s.ip] = s.ira[s.ip1] + s.ira[s.ip2];
    s.ip++; s.ip1++; s.ip2++; s.ip3++;
  }
  for (int i = 0; i < 1111; i++) or_hq_next(&s);
  *u = s;
}

/* Luescher RANLUX-24 used only for seeding (random_generator.cu:5-91). */
typedef struct { uint32_t v[256]; uint32_t carry; uint8_t ip, ip1, ip2; } luscher;

/* luxury(): 389 subtract-with-borrow steps per output, random_generator.cu:57-75 */
static uint32_t or_lus_next_(luscher *l) {
  for (int i = 0; i < 389; i++) {
    int32_t d = (int32_t)(l->v[l->ip1] - l->v[l->ip2] - l->carry);
    l->v[l->ip] = (uint32_t)((d + 16777216) & 16777215);
    l->carry = ((uint32_t)d) >> 31;
    l->ip++; l->ip1++; l->ip2++;
  }
  return l->v[l->ip];
}

/* Init_luxury, random_generator.cu:27-55 */
static void lus_init(luscher *l, uint64_t seed) {
  l->ip = 128; l->ip1 = 128 - 10; l->ip2 = 128 - 24;
  for (int i = 0; i < 1111; i++) seed = seed * LCG_A + 1;
  for (int j = l->ip2; j < l->ip; j++) {
    uint64_t t = 0;
    for (int i = 0; i < 3; i++) {
      seed = seed * LCG_A + 1;
      t |= (seed >> 56) << (8 * i);
    }
    l->v[j] = (uint32_t)t;
  }
  seed = seed * LCG_A + 1;
  l->carry = (uint32_t)(seed >> 63);
  for (int i = 0; i < 1111; i++) or_lus_next_(l);
}

/* Luescher_PRNG: top byte of 8 consecutive outputs, random_generator.cu:77-91 */
static uint64_t lus_u64(luscher *l) {
  uint64_t out = 0;
  for (int j = 0; j < 8; j++) out |= ((uint64_t)or_lus_next_(l) >> 16) << (8 * j);
  return out;
}

/* Inicia_generadores_CPU, random_generator.cu:94-158 */
void or_inicia_generadores(or_hq *prc, or_xo *xo, uint32_t *key, uint64_t seed) {
  luscher l;
  or_hq s;
  memset(&s, 0, sizeof(s));
  lus_init(&l, seed);
  for (int i = 0; i < 1111; i++) or_lus_next_(&l);
  s.zseed = lus_u64(&l);
  for (int k = 128 - 61; k < 128; k++) s.ira[k] = lus_u64(&l);
  s.ip = 128; s.ip1 = 128 - 24; s.ip2 = 128 - 55; s.ip3 = 128 - 61;
  for (int i = 0; i < 2222; i++) or_hq_next(&s);
  *prc = s;
  uint64_t st[4] = {0, 0, 0, 0};
  while (!(st[0] | st[1] | st[2] | st[3])) {
    for (int j = 0; j < 4; j++) {
      st[j] = 0;
      for (int i = 0; i < 64; i++) st[j] |= (((uint64_t)or_lus_next_(&l) >> 23) & 1ULL) << i;
    }
  }
  memset(xo, 0, sizeof(*xo));
  for (int j = 0; j < 4; j++) xo->s[j] = st[j];
  uint32_t k = 0;
  for (int i = 0; i < 32; i++) k |= ((or_lus_next_(&l) >> 23) & 1U) << i;
  *key = k;
}

/* generate_seeds_from_one, random_generator.cu:203-241 */
void or_seeds_from_one(uint64_t seed, uint64_t *list, int nseeds) {
  luscher l;
  lus_init(&l, seed);
  for (int i = 0; i < 1109; i++) or_lus_next_(&l);
  for (int s = 0; s < nseeds; s++) {
    uint64_t t = lus_u64(&l);
    t += LCG_A + 1;
    t >>= 62;
    static const int paranoia[4] = {709, 109, 1373, 2099};
    for (int i = 0; i < paranoia[t]; i++) or_lus_next_(&l);
    t = lus_u64(&l);
    list[s] = t * 6364136223846793005ULL + 14426950408889634071ULL;
  }
}

/* generate_seed_vectors, PROGRAM/src/ini.c:32-59 (MAXNSAMPLES = 32) */
void or_generate_seed_vectors(uint64_t master_J, uint64_t master_u, uint64_t master_MC,
                              const int *list_samples, int nbits, int NR, or_seeds *out) {
  uint64_t tmp[64];
  memset(out->seeds_J, 0, sizeof(out->seeds_J));
  memset(out->seeds_u, 0, sizeof(out->seeds_u));
  or_seeds_from_one(master_J, tmp, 32);
  for (int i = 0; i < nbits; i++) out->seeds_J[i] = tmp[list_samples[i]];
  or_seeds_from_one(master_u, tmp, 32);
  for (int i = 0; i < nbits; i++) out->seeds_u[i] = tmp[list_samples[i]];
  or_seeds_from_one(master_MC, tmp, NR);
  for (int r = 0; r < NR; r++) out->seeds_MC[r] = tmp[r];
}

/* Init_Random, PROGRAM/src/ini.c:61-101.  The per-sample PT seed passes through
 * an `int` (ini.c:63,90), so it is the low 32 bits sign-extended to 64. */
void or_init_random(const or_seeds *sd, const int *list_samples, int nbits, int NR,
                    or_hq *prc, or_xo *xo, uint32_t *keys, or_hq *pt, or_hq *rc) {
  uint64_t tmp[32];
  or_hq_init(rc, sd->seed_cluster);
  for (int r = 0; r < NR; r++) or_inicia_generadores(&prc[r], &xo[r], &keys[r], sd->seeds_MC[r]);
  for (int r = 0; r < NR; r++) {
    or_seeds_from_one(sd->seeds_MC[r], tmp, 32);
    for (int i = 0; i < nbits; i++) {
      int32_t s32 = (int32_t)(uint32_t)tmp[list_samples[i]];
      or_hq_init(&pt[i * NR + r], (uint64_t)(int64_t)s32);
    }
  }
}

/* ------------------------------------------------------------------------- */
/* Geometry tables: Init_MSC_neighbours + Init_MSC_index_and_rotate,          */
/* PROGRAM/src/ini.c:134-299.  The greedy split there yields the even-parity  */
/* MSC sites in index order ("bianchi") and the odd ones ("neri"); a site of  */
/* either colour sits at half index m>>1.                                     */
/* ------------------------------------------------------------------------- */
void or_tables(const or_geom *g, int32_t *neig, uint8_t *rot, uint32_t *bianchi, uint32_t *neri) {
  const int ml = g->msc_l, mlz = g->msc_lz, ms = g->msc_s, half = g->half;
  int nb = 0, nn = 0;
  for (int m = 0; m < g->msc_v; m++) {
    int a = m % ml, b = (m / ml) % ml, c = m / ms;
    if (((a + b + c) & 1) == 0) bianchi[nb++] = (uint32_t)m; else neri[nn++] = (uint32_t)m;
  }
  const int off[3] = {1, ml, ms};
  const int side[3] = {ml, ml, mlz};
  for (int p = 0; p < 2; p++) {
    const uint32_t *self = p ? neri : bianchi;
    for (int k = 0; k < half; k++) {
      int m = (int)self[k];
      int x[3] = {m % ml, (m / ml) % ml, m / ms};
      uint8_t rf = 0;
      for (int d = 0; d < 6; d++) {
        int dim = d % 3, sgn = d < 3 ? 1 : -1;
        int y[3] = {x[0], x[1], x[2]};
        y[dim] = (x[dim] + sgn + side[dim]) % side[dim];
        int mn = y[0] + y[1] * ml + y[2] * ms;
        neig[(p * 6 + d) * half + k] = mn >> 1;
        if (mn - m != sgn * off[dim]) rf |= (uint8_t)(1u << d);
      }
      rot[p * half + k] = rf;
    }
  }
}

/* Init_u, PROGRAM/src/ini.c:316-337 */
void or_init_spins(const or_geom *g, uint64_t seed_u, uint8_t *uu) {
  or_hq r;
  or_hq_init(&r, seed_u);
  size_t n = (size_t)g->NR * g->NB * g->V;
  for (size_t i = 0; i < n; i++) uu[i] = (uint8_t)(or_hq_next(&r) >> 63);
}

/* packing_u, PROGRAM/src/ini.c:339-383: bit bx+4by+16bz of word
 * [parity][clone][half][rep] holds site (alpha+bx*L/4, beta+by*L/4, gamma+bz*Lz/4). */
void or_pack_spins(const or_geom *g, const uint8_t *uu, uint64_t *even, uint64_t *odd) {
  const int L = g->L, Lz = g->Lz, ml = g->msc_l, mlz = g->msc_lz, NR = g->NR;
  size_t nw = (size_t)g->NB * g->half * NR;
  memset(even, 0, nw * 8); memset(odd, 0, nw * 8);
  uint64_t *w[2] = {even, odd};
  for (int r = 0; r < NR; r++)
    for (int c = 0; c < g->NB; c++) {
      const uint8_t *u = uu + ((size_t)r * g->NB + c) * g->V;
      int site = 0;
      for (int z = 0; z < Lz; z++)
        for (int y = 0; y < L; y++)
          for (int x = 0; x < L; x++, site++) {
            int bz = z / mlz, gam = z - bz * mlz, by = y / ml, bet = y - by * ml, bx = x / ml, al = x - bx * ml;
            int par = (x ^ y ^ z) & 1, bit = bx + 4 * by + 16 * bz;
            int ms = (al + ml * bet + gam * g->msc_s) / 2;
            size_t t = (size_t)r + (size_t)NR * ms + (size_t)g->half * NR * c;
            w[par][t] |= ((uint64_t)u[site]) << bit;
          }
    }
}

/* unpacking_u, PROGRAM/src/ini.c:385-433 */
void or_unpack_spins(const or_geom *g, const uint64_t *even, const uint64_t *odd, uint8_t *uu) {
  const int L = g->L, ml = g->msc_l, mlz = g->msc_lz, NR = g->NR, S = L * L;
  const uint64_t *w[2] = {even, odd};
  size_t nw = (size_t)g->NB * g->half * NR;
  for (size_t tid = 0; tid < nw; tid++) {
    int c = (int)(tid / ((size_t)g->half * NR));
    int rest = (int)(tid - (size_t)c * g->half * NR);
    int ms = rest / NR, r = rest - ms * NR;
    ms *= 2;
    int gam = ms / g->msc_s, re = ms - gam * g->msc_s, bet = re / ml, al = re - bet * ml;
    int bit = 0;
    uint8_t *u = uu + ((size_t)r * g->NB + c) * g->V;
    for (int bz = 0; bz < 4; bz++) {
      int z = bz * mlz + gam;
      for (int by = 0; by < 4; by++) {
        int y = by * ml + bet;
        for (int bx = 0; bx < 4; bx++, bit++) {
          int aux = bx * ml + al;
          for (int par = 0; par < 2; par++) {
            int x = aux | (par ^ ((y ^ z) & 1));
            u[x + y * L + z * S] = (uint8_t)((w[par][tid] >> bit) & 1);
          }
        }
      }
    }
  }
}

/* Init_J (random couplings), PROGRAM/src/ini.c:465-670.
 * J6 planes: 0 Jx, 1 Jy, 2 Jz, 3 Jmx, 4 Jmy, 5 Jmz.  Returns countJ. */
int or_init_couplings(const or_geom *g, uint64_t seed_J, uint8_t *J6) {
  const int L = g->L, Lz = g->Lz, V = g->V, S = L * L;
  uint8_t *Jx = J6, *Jy = J6 + V, *Jz = J6 + 2 * V, *Jmx = J6 + 3 * V, *Jmy = J6 + 4 * V, *Jmz = J6 + 5 * V;
  uint8_t *fz0 = (uint8_t *)calloc((size_t)V, 1);
  or_hq r;
  or_hq_init(&r, seed_J);
  int count = 0;
  for (int s = 0; s < V; s++) {
    Jx[s] = (uint8_t)(or_hq_next(&r) >> 63); count += Jx[s];
    Jy[s] = (uint8_t)(or_hq_next(&r) >> 63); count += Jy[s];
    Jz[s] = (uint8_t)(or_hq_next(&r) >> 63); count += Jz[s];
  }
  const int obc = g->bc != OR_PBC;
  if (obc) {
    for (int s = 0; s < S; s++) fz0[s] = (uint8_t)(or_hq_next(&r) >> 63);
    if (g->bc == OR_OBC_WEAK || g->bc == OR_OBC_STRONG) {
      uint8_t x1 = g->bc == OR_OBC_WEAK ? 1 : 0;
      for (int y = 0; y < L; y++)
        for (int x = 0; x < L; x++) {
          int s = x + y * L;
          if (((x ^ y) & 1) == 0) fz0[s] = Jy[s] ^ x1;
        }
      int z = Lz - 1;
      for (int y = 0; y < L; y++)
        for (int x = 0; x < L; x++) {
          int s = z * S + x + y * L;
          if (((x ^ y ^ z) & 1) == 0) Jz[s] = Jy[s] ^ x1;
        }
    }
    /* odd sites of the two boundary planes share the fake bond of their y-1 neighbour */
    for (int y = 0; y < L; y++) {
      int ym = y == 0 ? (L - 1) * L : -L;
      for (int x = 0; x < L; x++) {
        int s = x + y * L;
        if ((x ^ y) & 1) fz0[s] = fz0[s + ym];
      }
    }
    int z = Lz - 1;
    for (int y = 0; y < L; y++) {
      int ym = y == 0 ? (L - 1) * L : -L;
      for (int x = 0; x < L; x++) {
        int s = z * S + x + y * L;
        if ((x ^ y ^ z) & 1) Jz[s] = Jz[s + ym];
      }
    }
  }
  int site = 0;
  for (int z = 0; z < Lz; z++)
    for (int y = 0; y < L; y++)
      for (int x = 0; x < L; x++, site++) {
        int xm = x == 0 ? L - 1 : -1, ym = y == 0 ? (L - 1) * L : -L, zm = z == 0 ? (Lz - 1) * S : -S;
        Jmx[site] = Jx[site + xm];
        Jmy[site] = Jy[site + ym];
        if (!obc || z > 0) Jmz[site] = Jz[site + zm];
        else Jmz[site] = fz0[site];
      }
  free(fz0);
  return count;
}

/* packing_J, PROGRAM/src/ini.c:672-730 -> Jw[parity][dir][half] */
void or_pack_couplings(const or_geom *g, const uint8_t *J6, uint64_t *Jw) {
  const int L = g->L, Lz = g->Lz, ml = g->msc_l, mlz = g->msc_lz, V = g->V;
  uint64_t *J = (uint64_t *)calloc((size_t)g->msc_v * 6, 8);
  int site = 0;
  for (int z = 0; z < Lz; z++)
    for (int y = 0; y < L; y++)
      for (int x = 0; x < L; x++, site++) {
        int bz = z / mlz, gam = z - bz * mlz, by = y / ml, bet = y - by * ml, bx = x / ml, al = x - bx * ml;
        int bit = bx + 4 * by + 16 * bz;
        int m = al + ml * bet + gam * g->msc_s;
        for (int d = 0; d < 6; d++) J[6 * m + d] |= ((uint64_t)(J6[d * V + site] & 1)) << bit;
      }
  for (int m = 0; m < g->msc_v; m++) {
    int a = m % ml, b = (m / ml) % ml, c = m / g->msc_s;
    int p = (a + b + c) & 1, k = m >> 1;
    for (int d = 0; d < 6; d++) Jw[((size_t)p * 6 + d) * g->half + k] = J[6 * m + d];
  }
  free(J);
}

/* ------------------------------------------------------------------------- */
/* Metropolis random words                                                    */
/* ------------------------------------------------------------------------- */
/* _fill_bits, PROGRAM/include/fill_bits.h:47-68 (52 entropy bits per replica,
 * 14 in .x above iter/parity, 7 in .y above iter>>15, 13 in .z, 18 in .w above
 * the 14-bit job id).  parity = iter & 1 because iter starts even and is
 * incremented after each half-sweep (main.cu:139,319,343). */
void or_fill_bits(or_hq *prc, or_xo *xo, int NR, uint64_t iter, uint32_t jobid, uint32_t *ctr) {
  uint64_t parity = iter & 1ULL;
  for (int r = 0; r < NR; r++) {
    or_xo_next(&xo[r]);
    or_hq_next(&prc[r]);
    uint64_t e = (prc[r].final + xo[r].final) >> 12;
    uint32_t y = (uint32_t)(iter >> 15);
    uint32_t x = (uint32_t)(((iter & 32767ULL) << 3) | (parity << 2));
    x |= (uint32_t)((e & 0x3FFFULL) << 18); e >>= 14;
    y |= (uint32_t)((e & 0x7FULL) << 25); e >>= 7;
    uint32_t z = (uint32_t)((e & 0x1FFFULL) << 19); e >>= 13;
    uint32_t w = ((uint32_t)(e << 14)) | jobid;
    ctr[4 * r + 0] = x; ctr[4 * r + 1] = y; ctr[4 * r + 2] = z; ctr[4 * r + 3] = w;
  }
}

static inline uint32_t mulhi32(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }

/* Philox4x32-10 round function as written in main.cu:996-1043 */
static void philox10(uint32_t v[4], uint32_t k0, uint32_t k1) {
  for (int i = 0; i < 10; i++) {
    if (i) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint32_t lo0 = 0xD2511F53u * v[0], hi0 = mulhi32(0xD2511F53u, v[0]);
    uint32_t lo1 = 0xCD9E8D57u * v[2], hi1 = mulhi32(0xCD9E8D57u, v[2]);
    uint32_t n0 = hi1 ^ v[1] ^ k0, n2 = hi0 ^ v[3] ^ k1;
    v[0] = n0; v[1] = lo1; v[2] = n2; v[3] = lo0;
  }
}

/* LUT search: smallest n with R < cum[n], capped at 255.  The bisection with
 * the 12-bit pre-search at main.cu:1063-1078 computes exactly this function of R
 * (create_LUT.c:87-217 checks it at every interval end). */
int or_lut_search(uint64_t R, const uint64_t *cum) {
  int lo = 0, hi = 255;
  if (!(R < cum[254])) return 255;
  while (lo < hi) { int mid = (lo + hi) >> 1; if (R < cum[mid]) hi = mid; else lo = mid + 1; }
  return lo;
}

/* d_gen_rndbits_cuda body for one thread, main.cu:1045-1147 */
void or_rnd_triple(const uint32_t ctr[4], uint32_t key, uint32_t tid, const uint64_t *cum, uint64_t out[3]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2] + tid, ctr[3]};
  uint32_t w[6];
  for (int j = 0; j < 6; j++) {
    uint32_t v[4] = {c[0], c[1], c[2], c[3]};
    philox10(v, tid, key);
    c[0]++; /* 6 calls: the internal-call field overflows into parity/iter bits, as in the reference */
    uint32_t h = v[0] ^ v[2], l = v[1] ^ v[3];
    uint32_t lsb[4];
    lsb[0] = ((v[1] << 17) | (v[0] >> 15)) ^ h ^ ((h << 21) | (l >> 11));
    lsb[1] = ((v[0] << 17) | (v[1] >> 15)) ^ l ^ (l << 21);
    lsb[2] = (h << 28) | (l >> 4);
    lsb[3] = (l << 28) | (h >> 4);
    uint32_t rot = (lsb[0] + v[1] + lsb[2] + v[3]) >> 27;
    uint32_t bb = 0;
    for (int q = 0; q < 4; q++) {
      uint64_t R = ((uint64_t)v[q] << 32) | lsb[q];
      bb |= (uint32_t)or_lut_search(R, cum) << (8 * q);
    }
    w[j] = rot ? ((bb << rot) | (bb >> (32 - rot))) : bb; /* rot 0 leaves the word unchanged */
  }
  out[0] = ((uint64_t)w[0] << 32) | w[1];
  out[1] = ((uint64_t)w[2] << 32) | w[3];
  out[2] = ((uint64_t)w[4] << 32) | w[5];
}

/* RotateE..RotateD, main.cu:1154-1190 */
static inline uint64_t rotE(uint64_t o) { return (o & 0x1111111111111111ull) << 3 | (o & ~0x1111111111111111ull) >> 1; }
static inline uint64_t rotN(uint64_t o) { return (o & 0x000F000F000F000Full) << 12 | (o & ~0x000F000F000F000Full) >> 4; }
static inline uint64_t rotU(uint64_t o) { return (o & 0x000000000000FFFFull) << 48 | (o & ~0x000000000000FFFFull) >> 16; }
static inline uint64_t rotO(uint64_t o) { return (o & 0x8888888888888888ull) >> 3 | (o & ~0x8888888888888888ull) << 1; }
static inline uint64_t rotS(uint64_t o) { return (o & 0xF000F000F000F000ull) >> 12 | (o & ~0xF000F000F000F000ull) << 4; }
static inline uint64_t rotD(uint64_t o) { return (o & 0xFFFF000000000000ull) >> 48 | (o & ~0xFFFF000000000000ull) << 16; }
static inline uint64_t rot_dir(int d, uint64_t o) {
  switch (d) { case 0: return rotE(o); case 1: return rotN(o); case 2: return rotU(o);
               case 3: return rotO(o); case 4: return rotS(o); default: return rotD(o); }
}
#define MASK_LZM1 (~0xFFFF000000000000ull) /* main.cu:1207 */
#define MASK_0 (~0x000000000000FFFFull)    /* main.cu:1206 */

/* The six (rotated, OBC-patched) neighbour words of target (p, k) in the other
 * parity array `other` ([half][NR] of one clone), main.cu:1436-1472. */
static void gather_nb(const or_geom *g, const int32_t *neig, const uint8_t *rot, int p, int k,
                      const uint64_t *other, int r, uint64_t nb[6]) {
  const int half = g->half, NR = g->NR;
  uint8_t rf = rot[p * half + k];
  for (int d = 0; d < 6; d++) {
    uint64_t w = other[(size_t)neig[(p * 6 + d) * half + k] * NR + r];
    if (rf & (1u << d)) w = rot_dir(d, w);
    nb[d] = w;
  }
  if (g->bc != OR_PBC) {
    int gamma = (2 * k) / g->msc_s;
    uint64_t aux = p == 0 ? nb[1] : nb[4];
    if (gamma == g->msc_lz - 1) nb[2] = (nb[2] & MASK_LZM1) | (aux & ~MASK_LZM1);
    if (gamma == 0) nb[5] = (nb[5] & MASK_0) | (aux & ~MASK_0);
  }
}

typedef struct { int32_t *neig; uint8_t *rot; int half; } tabcache;

static void get_tables(const or_geom *g, int32_t **neig, uint8_t **rot) {
  *neig = (int32_t *)malloc(sizeof(int32_t) * 12 * g->half);
  *rot = (uint8_t *)malloc(2 * g->half);
  uint32_t *bi = (uint32_t *)malloc(4 * g->half), *ne = (uint32_t *)malloc(4 * g->half);
  or_tables(g, *neig, *rot, bi, ne);
  free(bi); free(ne);
}

/* Metropolis flip mask, main.cu:1474-1506 */
static inline uint64_t flip_mask(uint64_t s, const uint64_t *J, const uint64_t nb[6], uint64_t b0, uint64_t b1, uint64_t b2) {
  uint64_t f0 = s ^ J[0] ^ nb[0], f1 = s ^ J[1] ^ nb[1], f2 = s ^ J[2] ^ nb[2];
  uint64_t k1 = f0 ^ f1, k2 = f0 & f1, j1 = k1 ^ f2, k3 = k1 & f2, j2 = k2 ^ k3;
  f0 = s ^ J[3] ^ nb[3]; f1 = s ^ J[4] ^ nb[4]; f2 = s ^ J[5] ^ nb[5];
  k1 = f0 ^ f1; k2 = f0 & f1; k3 = k1 & f2;
  uint64_t j3 = k1 ^ f2, j4 = k2 ^ k3;
  b1 = b0 & b1; b2 = b1 & b2;
  uint64_t id2 = b1, id1 = (b0 ^ b1) | b2, j24 = j2 | j4;
  return (j1 & j3 & id1) | ((j24 | id2) & (j1 | j3 | id1)) | ((j2 & j4) | (j24 & id2));
}

void or_half_sweep(const or_geom *g, uint64_t *spins, const uint64_t *Jw, const uint8_t *wbtc,
                   const uint32_t *ctr, const uint32_t *keys, const uint64_t *cum, int parity, int nthreads) {
  const int NB = g->NB, NR = g->NR, half = g->half;
  const size_t nwc = (size_t)half * NR;          /* words per clone */
  const size_t nwp = nwc * NB;                     /* words per parity */
  int32_t *neig; uint8_t *rot;
  get_tables(g, &neig, &rot);
  /* random words: shared by all samples, indexed by beta (main.cu:1112-1147,1428-1430) */
  uint64_t *rnd = (uint64_t *)malloc(sizeof(uint64_t) * 3 * nwp);
  const long ntrip = (long)nwp;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
  for (long t = 0; t < ntrip; t++) {
    int beta = (int)(t / nwc), r = (int)(t % NR);
    or_rnd_triple(&ctr[4 * r], keys[r], (uint32_t)t, cum + 256 * beta, &rnd[3 * t]);
  }
  const long nwork = (long)g->nbits * NB * half;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (long w = 0; w < nwork; w++) {
    int s = (int)(w / ((long)NB * half));
    int c = (int)((w / half) % NB);
    int k = (int)(w % half);
    uint64_t *base = spins + (size_t)s * 2 * nwp;
    uint64_t *tgt = base + (size_t)parity * nwp + (size_t)c * nwc;
    const uint64_t *oth = base + (size_t)(1 - parity) * nwp + (size_t)c * nwc;
    const uint64_t *Jsp = Jw + ((size_t)s * 2 + parity) * 6 * half;
    uint64_t J[6];
    for (int d = 0; d < 6; d++) J[d] = Jsp[d * half + k];
    for (int r = 0; r < NR; r++) {
      int beta = wbtc[((size_t)s * NR + r) * NB + c];
      const uint64_t *b = &rnd[3 * ((size_t)beta * nwc + (size_t)k * NR + r)];
      uint64_t nb[6];
      gather_nb(g, neig, rot, parity, k, oth, r, nb);
      uint64_t sv = tgt[(size_t)k * NR + r];
      tgt[(size_t)k * NR + r] = sv ^ flip_mask(sv, J, nb, b[0], b[1], b[2]);
    }
  }
  free(rnd); free(neig); free(rot);
}

static inline int pop64(uint64_t x) { return __builtin_popcountll(x); }

/* d_computeEne over the even words, main.cu:1209-1381 */
void or_energy(const or_geom *g, const uint64_t *spins, const uint64_t *Jw, int32_t *E) {
  const int NB = g->NB, NR = g->NR, half = g->half;
  const size_t nwc = (size_t)half * NR, nwp = nwc * NB;
  int32_t *neig; uint8_t *rot;
  get_tables(g, &neig, &rot);
  for (int s = 0; s < g->nbits; s++)
    for (int r = 0; r < NR; r++)
      for (int c = 0; c < NB; c++) {
        const uint64_t *ev = spins + (size_t)s * 2 * nwp + (size_t)c * nwc;
        const uint64_t *od = ev + nwp;
        const uint64_t *Jsp = Jw + (size_t)s * 2 * 6 * half;
        int32_t e = 0;
        for (int k = 0; k < half; k++) {
          uint64_t nb[6];
          gather_nb(g, neig, rot, 0, k, od, r, nb);
          uint64_t sv = ev[(size_t)k * NR + r];
          int le = 0;
          for (int d = 0; d < 6; d++) le += pop64(sv ^ Jsp[d * half + k] ^ nb[d]);
          e += 6 * 64 - 2 * le;
        }
        E[((size_t)s * NR + r) * NB + c] = e;
      }
  free(neig); free(rot);
}

/* calculate_scalar_energy, PROGRAM/src/med.c:3-44 */
int or_scalar_energy(const or_geom *g, const uint8_t *u, const uint8_t *J6) {
  const int L = g->L, Lz = g->Lz, V = g->V, S = L * L;
  const uint8_t *Jx = J6, *Jy = J6 + V, *Jz = J6 + 2 * V, *Jmz = J6 + 5 * V;
  int e = 0, site = 0;
  for (int z = 0; z < Lz; z++)
    for (int y = 0; y < L; y++)
      for (int x = 0; x < L; x++, site++) {
        int par = (x ^ y ^ z) & 1;
        int px = x == L - 1 ? -(L - 1) : 1, py = y == L - 1 ? -(L - 1) * L : L, pz = z == Lz - 1 ? -(Lz - 1) * S : S;
        int sp = u[site];
        e += sp ^ Jx[site] ^ u[site + px];
        e += sp ^ Jy[site] ^ u[site + py];
        if (g->bc == OR_PBC) {
          e += sp ^ Jz[site] ^ u[site + pz];
        } else if (z == Lz - 1) {
          if (par == 0) e += sp ^ Jz[site] ^ u[site + py];
        } else {
          e += sp ^ Jz[site] ^ u[site + pz];
          if (z == 0 && par == 0) e += sp ^ Jmz[site] ^ u[site + py];
        }
      }
  return 3 * V - 2 * e;
}

/* Parallel_Tempering, PROGRAM/src/upd.c:3-48 (FNORM from random_generator.h:24) */
void or_parallel_tempering(or_hq *p, uint8_t *wctb, uint8_t *wbtc, const int32_t *E,
                           const double *betas, int NB, double *acc, double *att, double *accraw) {
  const double FNORM = 5.4210108624275218e-20;
  for (int i = 0; i < NB - 1; i++) {
    att[i]++;
    double pt = -(betas[i + 1] - betas[i]) * (double)(E[wctb[i + 1]] - E[wctb[i]]);
    or_hq_next(p);
    int change = 0;
    if (pt >= 0) { acc[i]++; change = 1; }
    else {
      double ex = exp(pt);
      acc[i] += ex;
      if ((FNORM * (double)p->final) < ex) change = 1;
    }
    if (change) { uint8_t t = wctb[i]; wctb[i] = wctb[i + 1]; wctb[i + 1] = t; accraw[i]++; }
  }
  for (int i = 0; i < NB; i++) wbtc[wctb[i]] = (uint8_t)i;
}

/* Replica pair of group g: partial Fisher-Yates with random_c, main.cu:409-421 */
void or_houdayer_pair(or_hq *rc, int NR, int g, int *r1, int *r2) {
  int h = NR / 2, idx[64];
  for (int k = 0; k < h; k++) idx[k] = k + g * h;
  for (int k = 0; k < h - 1; k++) {
    or_hq_next(rc);
    int j = k + (int)(((uint32_t)(rc->final >> 32)) % (uint32_t)(h - k));
    int t = idx[k]; idx[k] = idx[j]; idx[j] = t;
  }
  *r1 = idx[0]; *r2 = idx[1];
}

static uint32_t uf_find(uint32_t *par, uint32_t i) {
  while (par[i] != i) { par[i] = par[par[i]]; i = par[i]; }
  return i;
}

/* Equal-overlap clusters (HoudayerXEA.cu:77-121 bonds, 233-331 labelling): sites
 * joined to their -x, -y (periodic) and -z neighbours (periodic under PBC, no
 * wrap under OBC) when the overlap bits agree.  Komura's labelling ends with
 * every site pointing at the smallest index of its cluster. */
void or_cluster_roots(const or_geom *g, const uint8_t *q, uint32_t *root, int ref_quirk) {
  const int L = g->L, Lz = g->Lz, S = L * L, V = g->V;
  /* HoudayerXEA.cu:96 forms (ltid-1+nx)%nx with a 32-bit ltid, so for site 0
   * the x-wrap bond is tested against site (2^32-1+L) mod L, while the union
   * (HoudayerXEA.cu:288, 64-bit index) still joins site 0 with site L-1. */
  const int xq = (int)(((1ULL << 32) - 1 + (uint64_t)L) % (uint64_t)L);
  for (int i = 0; i < V; i++) root[i] = (uint32_t)i;
  for (int i = 0; i < V; i++) {
    int x = i % L, y = (i / L) % L, z = i / S;
    int nb[3], tst[3];
    nb[0] = (x == 0 ? L - 1 : x - 1) + y * L + z * S;
    nb[1] = x + (y == 0 ? L - 1 : y - 1) * L + z * S;
    nb[2] = (g->bc != OR_PBC && z == 0) ? -1 : x + y * L + (z == 0 ? Lz - 1 : z - 1) * S;
    tst[0] = (i == 0 && ref_quirk) ? xq : nb[0];
    tst[1] = nb[1]; tst[2] = nb[2];
    for (int d = 0; d < 3; d++) {
      if (nb[d] < 0 || q[tst[d]] != q[i]) continue;
      uint32_t a = uf_find(root, (uint32_t)i), b = uf_find(root, (uint32_t)nb[d]);
      if (a < b) root[b] = a; else if (b < a) root[a] = b;
    }
  }
  for (int i = 0; i < V; i++) root[i] = uf_find(root, (uint32_t)i);
}

/* d_computeoverlap + d_unpack + ClusterStep + d_pack + d_useoverlap,
 * main.cu:776-991 and HoudayerXEA.cu:54-75,183-211,358-374 */
void or_houdayer_group(const or_geom *g, uint64_t *spins, const uint8_t *wctb, int r1, int r2,
                       const double *U, int nclust, int ref_quirk) {
  const int NB = g->NB, NR = g->NR, half = g->half, V = g->V;
  const size_t nwc = (size_t)half * NR, nwp = nwc * NB;
  uint8_t *q = (uint8_t *)malloc((size_t)V);
  uint8_t *uu = (uint8_t *)malloc((size_t)NR * NB * V);
  uint32_t *root = (uint32_t *)malloc(sizeof(uint32_t) * V);
  or_geom g1 = *g; g1.NB = 1; g1.NR = 1;
  uint64_t *qe = (uint64_t *)malloc(8 * half), *qo = (uint64_t *)malloc(8 * half);
  uint8_t *qu = (uint8_t *)malloc((size_t)V);
  for (int s = 0; s < g->nbits; s++) {
    uint64_t *ev = spins + (size_t)s * 2 * nwp, *od = ev + nwp;
    for (int b = 0; b < nclust && b < NB; b++) {
      int c1 = wctb[((size_t)s * NR + r1) * NB + b], c2 = wctb[((size_t)s * NR + r2) * NB + b];
      for (int k = 0; k < half; k++) {
        qe[k] = ev[(size_t)c1 * nwc + (size_t)k * NR + r1] ^ ev[(size_t)c2 * nwc + (size_t)k * NR + r2];
        qo[k] = od[(size_t)c1 * nwc + (size_t)k * NR + r1] ^ od[(size_t)c2 * nwc + (size_t)k * NR + r2];
      }
      or_unpack_spins(&g1, qe, qo, qu);
      memcpy(q, qu, (size_t)V);
      or_cluster_roots(g, q, root, ref_quirk);
      const double *Ub = U + ((size_t)s * NB + b) * V;
      for (int i = 0; i < V; i++) qu[i] = q[i] ^ (uint8_t)(Ub[root[i]] < 0.5);
      or_pack_spins(&g1, qu, qe, qo);
      for (int k = 0; k < half; k++) {
        ev[(size_t)c1 * nwc + (size_t)k * NR + r1] ^= qe[k];
        ev[(size_t)c2 * nwc + (size_t)k * NR + r2] ^= qe[k];
        od[(size_t)c1 * nwc + (size_t)k * NR + r1] ^= qo[k];
        od[(size_t)c2 * nwc + (size_t)k * NR + r2] ^= qo[k];
      }
    }
  }
  free(q); free(uu); free(root); free(qe); free(qo); free(qu);
}

/* ------------------------------------------------------------------------- */
/* LUT, PROGRAM/input/create_LUT.c:265-388                                    */
/* ------------------------------------------------------------------------- */
int or_lut_beta(double beta, int nbits_pre, uint64_t *cum, uint32_t *umb, uint32_t *pre) {
#ifdef OR_HAVE_QUADMATH
  __float128 qb = (__float128)beta;
  __float128 p0 = (1.0Q - expq(-4.0Q * qb)), p1 = expq(-4.0Q * qb);
  uint64_t caso[9];
  for (int i = 0; i < 9; i++) {
    __float128 pr = powq(p0, 8 - i) * powq(p1, i);
    __float128 t = 18446744073709551616.Q * pr;
    caso[i] = (uint64_t)t;
  }
  cum[0] = caso[0];
  for (int i = 1; i < 255; i++) cum[i] = cum[i - 1] + caso[__builtin_popcount(i)];
  cum[255] = ~0ULL;
  for (int i = 0; i < 256; i++) { umb[2 * i] = (uint32_t)(cum[i] >> 32); umb[2 * i + 1] = (uint32_t)cum[i]; }
  int npre = 1 << nbits_pre;
  uint64_t tail = (1ULL << (64 - nbits_pre)) - 1ULL;
  uint32_t *tmin = (uint32_t *)malloc(4 * npre), *tmax = (uint32_t *)malloc(4 * npre);
  for (int m = 0; m < npre; m++) {
    uint64_t t = (uint64_t)m << (64 - nbits_pre);
    int i;
    for (i = 0; i < 256; i++) if (t < cum[i]) break;
    tmin[m] = (uint32_t)(i > 255 ? 255 : i);
    t |= tail;
    for (i = 0; i < 256; i++) if (t < cum[i]) break;
    tmax[m] = (uint32_t)(i > 255 ? 255 : i);
  }
  for (int i = 0; i < npre; i += 8)
    for (int j = 0; j < 4; j++)
      pre[(i >> 3) * 4 + j] = tmin[i + 2 * j] | (tmax[i + 2 * j] << 8) | (tmin[i + 2 * j + 1] << 16) | (tmax[i + 2 * j + 1] << 24);
  free(tmin); free(tmax);
  return 0;
#else
  (void)beta; (void)nbits_pre; (void)cum; (void)umb; (void)pre;
  return -1;
#endif
}

/* ------------------------------------------------------------------------- */
/* One bin of the driver loop, PROGRAM/src/main.cu:142-230, 285-349, 351-453, 531-554 */
/* ------------------------------------------------------------------------- */
int or_run_bin(or_state *st, const or_run_cfg *cfg, uint64_t *iter) {
  or_geom *g = &st->g;
  const int NB = g->NB, NR = g->NR, nbits = g->nbits;
  uint32_t *ctr = (uint32_t *)malloc(16 * NR);
  for (int s = 0; s < nbits; s++) memset(st->avgE + (size_t)s * NR * NB, 0, sizeof(double) * NR * NB);
  double *U = NULL;
  size_t totrandom = (size_t)g->V * NB * nbits;
  if (cfg->cluster) U = (double *)malloc(sizeof(double) * totrandom);
  for (int it = 0; it < cfg->itmax; it++) {
    for (int imes = 0; imes < cfg->mesfr; imes++) {
      for (int ihou = 0; ihou < cfg->houfr; ihou++) {
        for (int im = 0; im < cfg->ptfr; im++) {
          for (int par = 0; par < 2; par++) {
            or_fill_bits(st->prc, st->xo, NR, *iter, cfg->jobid, ctr);
            or_half_sweep(g, st->spins, st->Jw, st->wbtc, ctr, st->keys, st->cum, par, cfg->nthreads);
            (*iter)++;
          }
        }
        or_energy(g, st->spins, st->Jw, st->E);
        for (int s = 0; s < nbits; s++)
          for (int r = 0; r < NR; r++) {
            size_t o = ((size_t)s * NR + r);
            or_parallel_tempering(&st->pt[o], st->wctb + o * NB, st->wbtc + o * NB, st->E + o * NB,
                                  st->betas, NB, st->acc + o * (NB - 1), st->att + o * (NB - 1),
                                  st->accraw + o * (NB - 1));
          }
      }
      if (cfg->cluster) {
        for (int gi = 0; gi < 2; gi++) {
          int r1, r2;
          or_houdayer_pair(&st->rc, NR, gi, &r1, &r2);
#ifdef OR_HAVE_CURAND
          if (!st->curand_gen) {
            curandGenerator_t gen;
            if (curandCreateGeneratorHost(&gen, CURAND_RNG_PSEUDO_DEFAULT) != CURAND_STATUS_SUCCESS) { free(ctr); free(U); return -2; }
            curandSetPseudoRandomGeneratorSeed(gen, (unsigned long long)st->seed_cluster);
            if (st->cuda_rng_offset > 0) curandSetGeneratorOffset(gen, st->cuda_rng_offset);
            st->curand_gen = (void *)gen;
          }
          if (curandGenerateUniformDouble((curandGenerator_t)st->curand_gen, U, totrandom) != CURAND_STATUS_SUCCESS) { free(ctr); free(U); return -2; }
#else
          free(ctr); free(U); return -2;
#endif
          st->cuda_rng_offset += totrandom;
          or_houdayer_group(g, st->spins, st->wctb, r1, r2, U, cfg->nclust, !cfg->cluster_exact);
        }
      }
    }
    or_energy(g, st->spins, st->Jw, st->E);
    for (int s = 0; s < nbits; s++)
      for (int r = 0; r < NR; r++)
        for (int b = 0; b < NB; b++) {
          size_t o = (size_t)s * NR + r;
          st->avgE[o * NB + b] += (double)st->E[o * NB + st->wctb[o * NB + b]];
        }
    if (it % st->frec_trw == st->frec_trw - 1) {
      int itm = it / st->frec_trw;
      for (int s = 0; s < nbits; s++)
        for (int r = 0; r < NR; r++) {
          size_t o = (size_t)s * NR + r;
          memcpy(st->hist + (o * st->maxit_trw + itm) * NB, st->wbtc + o * NB, NB);
        }
    }
  }
  free(ctr); free(U);
  return 0;
}

/* cuRAND XORWOW host generator (the library the reference calls on the device,
 * HoudayerXEA.cu:174-178,189): n uniform doubles at seed/offset. */
int or_curand_host(uint64_t seed, uint64_t offset, uint64_t n, double *out) {
#ifdef OR_HAVE_CURAND
  curandGenerator_t gen;
  if (curandCreateGeneratorHost(&gen, CURAND_RNG_PSEUDO_DEFAULT) != CURAND_STATUS_SUCCESS) return -2;
  curandSetPseudoRandomGeneratorSeed(gen, (unsigned long long)seed);
  if (offset) curandSetGeneratorOffset(gen, offset);
  curandStatus_t s = curandGenerateUniformDouble(gen, out, n);
  curandDestroyGenerator(gen);
  return s == CURAND_STATUS_SUCCESS ? 0 : -2;
#else
  (void)seed; (void)offset; (void)n; (void)out;
  return -2;
#endif
}

void or_state_release(or_state *st) {
#ifdef OR_HAVE_CURAND
  if (st->curand_gen) curandDestroyGenerator((curandGenerator_t)st->curand_gen);
#endif
  st->curand_gen = NULL;
}
