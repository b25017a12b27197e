// host.cpp -- job set-up on the host: generator seeding, geometry tables,
// initial spins and couplings, multispin packing, PT exp table.
//
// Each piece follows the reference's host code (paths relative to the
// reference project): PROGRAM/src/random_generator.cu, PROGRAM/src/ini.c,
// PROGRAM/src/med.c, PROGRAM/src/upd.c.
#include "host.hpp"

#include <cmath>
#include <cstring>

namespace eagb {

// Init_Rand_HQ_64bits (random_generator.cu:160-201): LCG warm-up, 61 lagged
// words from the LCG's top bytes, 1111 plain Fibonacci steps, 1111 full steps.
void hq_seed(ea_hq &u, uint64_t seed) {
  ea_hq s;
  std::memset(&s, 0, sizeof(s));
  s.zseed = seed;
  for (int i = 0; i < 111; ++i) s.zseed = s.zseed * kLcg + 1;
  for (int k = 67; k < 128; ++k) {
    uint64_t w = 0;
    for (int i = 0; i < 8; ++i) {
      s.zseed = s.zseed * kLcg + 1;
      w |= (s.zseed >> 56) << (8 * i);
    }
    s.ira[k] = w;
  }
  s.ip = 128; s.ip1 = 104; s.ip2 = 73; s.ip3 = 67;
  for (int i = 0; i < 1111; ++i) {
    s.ira[s.ip] = s.ira[s.ip1] + s.ira[s.ip2];
    ++s.ip; ++s.ip1; ++s.ip2; ++s.ip3;
  }
  for (int i = 0; i < 1111; ++i) hq_next(s);
  u = s;
}

namespace {

// 24-bit subtract-with-borrow generator with luxury level 389, used only to
// derive seeds (random_generator.cu:5-91).
class Ranlux24 {
 public:
  explicit Ranlux24(uint64_t seed) {
    for (int i = 0; i < 1111; ++i) seed = seed * kLcg + 1;
    for (int j = p2_; j < p0_; ++j) {
      uint64_t t = 0;
      for (int i = 0; i < 3; ++i) {
        seed = seed * kLcg + 1;
        t |= (seed >> 56) << (8 * i);
      }
      v_[j] = (uint32_t)t;
    }
    seed = seed * kLcg + 1;
    borrow_ = (uint32_t)(seed >> 63);
    discard(1111);
  }
  uint32_t next() {
    for (int i = 0; i < 389; ++i) {
      int32_t d = (int32_t)(v_[p1_] - v_[p2_] - borrow_);
      v_[p0_] = (uint32_t)((d + (1 << 24)) & ((1 << 24) - 1));
      borrow_ = (uint32_t)d >> 31;
      ++p0_; ++p1_; ++p2_;
    }
    return v_[p0_];
  }
  void discard(int n) { for (int i = 0; i < n; ++i) next(); }
  uint64_t next_u64() {  // Luescher_PRNG: top byte of eight outputs
    uint64_t o = 0;
    for (int j = 0; j < 8; ++j) o |= ((uint64_t)next() >> 16) << (8 * j);
    return o;
  }
  uint32_t bit23() { return (next() >> 23) & 1u; }

 private:
  uint32_t v_[256] = {};
  uint32_t borrow_ = 0;
  uint8_t p0_ = 128, p1_ = 118, p2_ = 104;
};

}  // namespace

// generate_seeds_from_one (random_generator.cu:203-241).
void seeds_from_one(uint64_t seed, uint64_t *out, int n) {
  static const int kSkip[4] = {709, 109, 1373, 2099};
  Ranlux24 r(seed);
  r.discard(1109);
  for (int s = 0; s < n; ++s) {
    uint64_t t = (r.next_u64() + kLcg + 1) >> 62;
    r.discard(kSkip[t]);
    out[s] = r.next_u64() * 6364136223846793005ULL + 14426950408889634071ULL;
  }
}

// Inicia_generadores_CPU (random_generator.cu:94-158).
void init_generators(uint64_t seed, ea_hq &prc, ea_xoshiro &xo, uint32_t &key) {
  Ranlux24 r(seed);
  r.discard(1111);
  ea_hq s;
  std::memset(&s, 0, sizeof(s));
  s.zseed = r.next_u64();
  for (int k = 67; k < 128; ++k) s.ira[k] = r.next_u64();
  s.ip = 128; s.ip1 = 104; s.ip2 = 73; s.ip3 = 67;
  for (int i = 0; i < 2222; ++i) hq_next(s);
  prc = s;
  uint64_t st[4] = {0, 0, 0, 0};
  while ((st[0] | st[1] | st[2] | st[3]) == 0) {
    for (int j = 0; j < 4; ++j) {
      st[j] = 0;
      for (int i = 0; i < 64; ++i) st[j] |= (uint64_t)r.bit23() << i;
    }
  }
  std::memset(&xo, 0, sizeof(xo));
  for (int j = 0; j < 4; ++j) xo.s[j] = st[j];
  uint32_t k = 0;
  for (int i = 0; i < 32; ++i) k |= r.bit23() << i;
  key = k;
}

bool Geometry::set(const ea_geom &g) {
  if (g.L < 8 || g.Lz < 8 || (g.L % 8) || (g.Lz % 8)) return false;
  if (g.nbetas < 2 || g.nbetas > 255 || g.nrep < 1 || g.nrep > 64 || g.nsamples < 1 || g.nsamples > 32) return false;
  if (g.bc < EA_PBC || g.bc > EA_OBC_STRONG) return false;
  L = g.L; Lz = g.Lz; NB = g.nbetas; NR = g.nrep; ns = g.nsamples; bc = g.bc;
  msc_l = L / 4; msc_lz = Lz / 4; msc_s = msc_l * msc_l; msc_v = msc_s * msc_lz;
  half = msc_v / 2; V = L * L * Lz;
  // The Philox counter reserves 19 bits for the thread index (fill_bits.h:9-20);
  // larger jobs still run (the index then overlaps entropy bits), as in the reference.
  return true;
}

// Init_MSC_neighbours + Init_MSC_index_and_rotate (ini.c:134-299): colour c of
// the (L/4)^2 (Lz/4) multispin lattice holds the sites of parity c in index order,
// so MSC site m sits at half index m >> 1.  A neighbour across the MSC wrap sits
// in the next spatial sub-block and its word is bit-rotated.
void neighbour_tables(const Geometry &g, std::vector<int32_t> &idx, std::vector<uint8_t> &flags) {
  idx.assign((size_t)12 * g.half, 0);
  flags.assign((size_t)2 * g.half, 0);
  const int side[3] = {g.msc_l, g.msc_l, g.msc_lz};
  const int off[3] = {1, g.msc_l, g.msc_s};
  for (int m = 0; m < g.msc_v; ++m) {
    int x[3] = {m % g.msc_l, (m / g.msc_l) % g.msc_l, m / g.msc_s};
    int p = (x[0] + x[1] + x[2]) & 1, k = m >> 1;
    uint8_t f = 0;
    for (int d = 0; d < 6; ++d) {
      int dim = d % 3, step = d < 3 ? 1 : -1;
      int y[3] = {x[0], x[1], x[2]};
      y[dim] = (x[dim] + step + side[dim]) % side[dim];
      int mn = y[0] + y[1] * g.msc_l + y[2] * g.msc_s;
      idx[((size_t)p * 6 + d) * g.half + k] = mn >> 1;
      if (mn - m != step * off[dim]) f |= (uint8_t)(1u << d);
    }
    if (x[2] == g.msc_lz - 1) f |= 0x40;
    if (x[2] == 0) f |= 0x80;
    flags[(size_t)p * g.half + k] = f;
  }
}

// Init_u (ini.c:316-337): one HQ draw per site, replica-major, clone, site order.
void init_spin_bytes(const Geometry &g, uint64_t seed_u, std::vector<uint8_t> &uu) {
  ea_hq r;
  hq_seed(r, seed_u);
  uu.resize((size_t)g.NR * g.NB * g.V);
  for (auto &b : uu) b = (uint8_t)(hq_next(r) >> 63);
}

// Bit bx + 4 by + 16 bz of word (clone, half, rep) holds the site
// (alpha + bx L/4, beta + by L/4, gamma + bz Lz/4) (ini.c:339-383).
void pack_clone(const Geometry &g, const uint8_t *u, int rep, int clone, uint64_t *even, uint64_t *odd) {
  const size_t base = (size_t)clone * g.words_per_clone() + rep;
  for (int k = 0; k < g.half; ++k) { even[base + (size_t)k * g.NR] = 0; odd[base + (size_t)k * g.NR] = 0; }
  int site = 0;
  for (int z = 0; z < g.Lz; ++z) {
    const int bz = z / g.msc_lz, gz = z % g.msc_lz;
    for (int y = 0; y < g.L; ++y) {
      const int by = y / g.msc_l, gy = y % g.msc_l;
      for (int x = 0; x < g.L; ++x, ++site) {
        const int bx = x / g.msc_l, gx = x % g.msc_l;
        const int m = gx + g.msc_l * gy + g.msc_s * gz;
        uint64_t *w = ((x ^ y ^ z) & 1) ? odd : even;
        w[base + (size_t)(m >> 1) * g.NR] |= (uint64_t)(u[site] & 1) << (bx + 4 * by + 16 * bz);
      }
    }
  }
}

void unpack_clone(const Geometry &g, const uint64_t *even, const uint64_t *odd, int rep, int clone, uint8_t *u) {
  const size_t base = (size_t)clone * g.words_per_clone() + rep;
  int site = 0;
  for (int z = 0; z < g.Lz; ++z) {
    const int bz = z / g.msc_lz, gz = z % g.msc_lz;
    for (int y = 0; y < g.L; ++y) {
      const int by = y / g.msc_l, gy = y % g.msc_l;
      for (int x = 0; x < g.L; ++x, ++site) {
        const int bx = x / g.msc_l, gx = x % g.msc_l;
        const int m = gx + g.msc_l * gy + g.msc_s * gz;
        const uint64_t *w = ((x ^ y ^ z) & 1) ? odd : even;
        u[site] = (uint8_t)((w[base + (size_t)(m >> 1) * g.NR] >> (bx + 4 * by + 16 * bz)) & 1);
      }
    }
  }
}

// Init_J, random couplings (ini.c:465-670).  Under OBC the z = 0 and z = Lz-1
// planes get "fake" bonds that join each even site to its y+1 neighbour; odd
// sites copy the coupling of their y-1 neighbour so both ends agree.
int init_couplings(const Geometry &g, uint64_t seed_J, uint8_t *J6) {
  const int L = g.L, Lz = g.Lz, V = g.V, S = L * L;
  uint8_t *Jx = J6, *Jy = J6 + V, *Jz = J6 + 2 * V, *Jmx = J6 + 3 * V, *Jmy = J6 + 4 * V, *Jmz = J6 + 5 * V;
  std::vector<uint8_t> fake(S, 0);
  ea_hq r;
  hq_seed(r, seed_J);
  int count = 0;
  for (int s = 0; s < V; ++s) {
    Jx[s] = (uint8_t)(hq_next(r) >> 63);
    Jy[s] = (uint8_t)(hq_next(r) >> 63);
    Jz[s] = (uint8_t)(hq_next(r) >> 63);
    count += Jx[s] + Jy[s] + Jz[s];
  }
  const bool obc = g.bc != EA_PBC;
  auto ym = [&](int y) { return y == 0 ? (L - 1) * L : -L; };
  if (obc) {
    for (int s = 0; s < S; ++s) fake[s] = (uint8_t)(hq_next(r) >> 63);
    if (g.bc == EA_OBC_WEAK || g.bc == EA_OBC_STRONG) {
      const uint8_t inv = g.bc == EA_OBC_WEAK;
      const int zt = Lz - 1;
      for (int y = 0; y < L; ++y)
        for (int x = 0; x < L; ++x) {
          if (((x ^ y) & 1) == 0) fake[x + y * L] = Jy[x + y * L] ^ inv;
          const int st = zt * S + x + y * L;
          if (((x ^ y ^ zt) & 1) == 0) Jz[st] = Jy[st] ^ inv;
        }
    }
    for (int y = 0; y < L; ++y)
      for (int x = 0; x < L; ++x)
        if ((x ^ y) & 1) fake[x + y * L] = fake[x + y * L + ym(y)];
    const int zt = Lz - 1;
    for (int y = 0; y < L; ++y)
      for (int x = 0; x < L; ++x) {
        const int st = zt * S + x + y * L;
        if ((x ^ y ^ zt) & 1) Jz[st] = Jz[st + ym(y)];
      }
  }
  int site = 0;
  for (int z = 0; z < Lz; ++z)
    for (int y = 0; y < L; ++y)
      for (int x = 0; x < L; ++x, ++site) {
        Jmx[site] = Jx[site + (x == 0 ? L - 1 : -1)];
        Jmy[site] = Jy[site + ym(y)];
        if (!obc || z > 0) Jmz[site] = Jz[site + (z == 0 ? (Lz - 1) * S : -S)];
        else Jmz[site] = fake[site];
      }
  return count;
}

// packing_J (ini.c:672-730): Jw[parity][dir][half].
void pack_couplings(const Geometry &g, const uint8_t *J6, uint64_t *Jw) {
  std::memset(Jw, 0, sizeof(uint64_t) * 12 * g.half);
  int site = 0;
  for (int z = 0; z < g.Lz; ++z)
    for (int y = 0; y < g.L; ++y)
      for (int x = 0; x < g.L; ++x, ++site) {
        const int bit = x / g.msc_l + 4 * (y / g.msc_l) + 16 * (z / g.msc_lz);
        const int m = x % g.msc_l + g.msc_l * (y % g.msc_l) + g.msc_s * (z % g.msc_lz);
        const int p = (x ^ y ^ z) & 1;
        for (int d = 0; d < 6; ++d)
          Jw[((size_t)p * 6 + d) * g.half + (m >> 1)] |= (uint64_t)(J6[(size_t)d * g.V + site] & 1) << bit;
      }
}

// calculate_scalar_energy (med.c:3-44), including the OBC fake bonds.
int scalar_energy(const Geometry &g, const uint8_t *u, const uint8_t *J6) {
  const int L = g.L, Lz = g.Lz, V = g.V, S = L * L;
  const uint8_t *Jx = J6, *Jy = J6 + V, *Jz = J6 + 2 * V, *Jmz = J6 + 5 * V;
  int e = 0, site = 0;
  for (int z = 0; z < Lz; ++z)
    for (int y = 0; y < L; ++y)
      for (int x = 0; x < L; ++x, ++site) {
        const int sp = u[site], even = ((x ^ y ^ z) & 1) == 0;
        const int px = x == L - 1 ? 1 - L : 1, py = y == L - 1 ? (1 - L) * L : L, pz = z == Lz - 1 ? (1 - Lz) * S : S;
        e += sp ^ Jx[site] ^ u[site + px];
        e += sp ^ Jy[site] ^ u[site + py];
        if (g.bc == EA_PBC) {
          e += sp ^ Jz[site] ^ u[site + pz];
        } else if (z == Lz - 1) {
          if (even) e += sp ^ Jz[site] ^ u[site + py];
        } else {
          e += sp ^ Jz[site] ^ u[site + pz];
          if (z == 0 && even) e += sp ^ Jmz[site] ^ u[site + py];
        }
      }
  return 3 * V - 2 * e;
}

void presearch8(const uint64_t *cum, uint16_t *pre) {
  auto first_above = [&](uint64_t R) {
    int n = 0;
    while (n < 255 && !(R < cum[n])) ++n;
    return n;
  };
  for (int b = 0; b < 256; ++b) {
    const uint64_t lo = (uint64_t)b << 56, hi = lo | ((1ULL << 56) - 1);
    pre[b] = (uint16_t)(first_above(lo) | (first_above(hi) << 8));
  }
}

// The 11-bit pre-search: pre[t] = the first byte n with (t << 53) < cum[n]
// for t < 2048 and 255 from entry 2048 on (kPre11Stride entries a
// temperature).  A key R in bucket t = R >> 53 has its byte in
// [pre[t], pre[t+1]]: the search is monotone in R, so the first byte of the
// next bucket bounds every byte of this one.
void presearch11(const uint64_t *cum, uint8_t *pre) {
  int n = 0;
  for (int t = 0; t < 2048; ++t) {
    const uint64_t lo = (uint64_t)t << 53;
    while (n < 255 && !(lo < cum[n])) ++n;
    pre[t] = (uint8_t)n;
  }
  for (int t = 2048; t < kPre11Stride; ++t) pre[t] = 255;
}

// pt = -(beta[i+1]-beta[i]) * dE in double, exactly as upd.c:16-17 forms it,
// and exp() from the host libm, as upd.c:29 calls it.  dE is even (E = 3V - 2n).
void pt_exp_table(const double *betas, int NB, std::vector<double> &vals, std::vector<int32_t> &offsets) {
  vals.clear();
  offsets.assign((size_t)NB, 0);
  const double kCut = -50.0;  // exp(-50) < 2^-72 < FNORM = 2^-64
  for (int i = 0; i + 1 < NB; ++i) {
    offsets[i] = (int32_t)vals.size();
    for (int32_t j = 1;; ++j) {
      const double dE = (double)(-2 * j);
      const double pt = -(betas[i + 1] - betas[i]) * dE;
      if (!(pt < 0) || pt < kCut || j > (1 << 22)) break;
      vals.push_back(std::exp(pt));
    }
  }
  offsets[NB - 1] = (int32_t)vals.size();
}

}  // namespace eagb
