// sp_host.cpp -- host side of the sample-packed layout: the tube's bond graph
// (neighbour slots, the fake bonds of the open z planes, half-edge mates), a
// proper colouring, and the seeded couplings and initial spins.
#include <algorithm>
#include <cstring>
#include <thread>

#include "host.hpp"
#include "sp.cuh"

namespace eagb {

namespace {

inline int site_of(const SpGraph &g, int x, int y, int z) { return x + g.L * (y + g.L * z); }

// Partner of a site of an open z plane through its fake bond.  The reference
// pairs each plane site with a y neighbour chosen by the parity of x+y+z
// (ini.c:551-641; the +y neighbour for even sites, -y for odd ones); that
// pairing needs L even.  For odd L the plane has an odd number of sites:
// sites pair along x (x even with x+1) up to column L-1, that column pairs
// along y (y even with y+1), and the last site (L-1, L-1) pairs with the same
// site of the other open plane.
void fake_partner(const SpGraph &g, int x, int y, int z, int &px, int &py, int &pz) {
  const int L = g.L;
  px = x; py = y; pz = z;
  if (L % 2 == 0) {
    py = ((x + y + z) & 1) ? (y + L - 1) % L : (y + 1) % L;
  } else if (x < L - 1) {
    px = (x & 1) ? x - 1 : x + 1;
  } else if (y < L - 1) {
    py = (y & 1) ? y - 1 : y + 1;
  } else {
    pz = z == 0 ? g.Lz - 1 : 0;
  }
}

bool proper(const SpGraph &g) {
  for (int i = 0; i < g.V; ++i)
    for (int d = 0; d < 6; ++d)
      if (g.colour[i] == g.colour[g.nb[i * 6 + d]]) return false;
  return true;
}

// colour of t on a cycle of n sites (periodic) or a chain, values in Z3: the
// parity, except the last site of an odd cycle
inline int cyc3(int t, int n, bool periodic) { return (periodic && (n & 1) && t == n - 1) ? 2 : (t & 1); }

}  // namespace

bool sp_graph(int L, int Lz, int bc, SpGraph &g) {
  if (L < 2 || Lz < 2 || L > 1024 || Lz > 65536 || (bc != EA_PBC && bc != EA_OBC)) return false;
  if ((long long)L * L * Lz > (1LL << 28)) return false;
  g.L = L; g.Lz = Lz; g.bc = bc; g.V = L * L * Lz;
  const int V = g.V;
  g.nb.assign((size_t)V * 6, 0);
  g.mate.assign((size_t)V * 6, 0);
  const bool obc = bc == EA_OBC;
  for (int z = 0; z < Lz; ++z)
    for (int y = 0; y < L; ++y)
      for (int x = 0; x < L; ++x) {
        const int i = site_of(g, x, y, z);
        int *n = &g.nb[(size_t)i * 6];
        int *m = &g.mate[(size_t)i * 6];
        n[0] = site_of(g, (x + 1) % L, y, z);
        n[1] = site_of(g, x, (y + 1) % L, z);
        n[2] = site_of(g, x, y, (z + 1) % Lz);
        n[3] = site_of(g, (x + L - 1) % L, y, z);
        n[4] = site_of(g, x, (y + L - 1) % L, z);
        n[5] = site_of(g, x, y, (z + Lz - 1) % Lz);
        for (int d = 0; d < 6; ++d) m[d] = n[d] * 6 + (d + 3) % 6;
        // the fake bond takes the slot of the missing z bond (+z on the top
        // plane, -z on the bottom one), at both of its ends
        if (obc && z == Lz - 1) {
          int px, py, pz;
          fake_partner(g, x, y, z, px, py, pz);
          const int p = site_of(g, px, py, pz);
          n[2] = p;
          m[2] = p * 6 + (pz == Lz - 1 ? 2 : 5);
        }
        if (obc && z == 0) {
          int px, py, pz;
          fake_partner(g, x, y, z, px, py, pz);
          const int p = site_of(g, px, py, pz);
          n[5] = p;
          m[5] = p * 6 + (pz == Lz - 1 ? 2 : 5);
        }
      }
  g.colour.assign((size_t)V, 0);
  bool ok = false;
  if (L % 2 == 0 && (obc || Lz % 2 == 0)) {
    g.ncol = 2;
    for (int i = 0; i < V; ++i) {
      const int x = i % L, y = (i / L) % L, z = i / (L * L);
      g.colour[i] = (uint8_t)((x + y + z) & 1);
    }
    ok = proper(g);
  }
  if (!ok) {
    g.ncol = 3;
    for (int i = 0; i < V; ++i) {
      const int x = i % L, y = (i / L) % L, z = i / (L * L);
      // z coloured as a cycle under OBC too: still proper on the open chain,
      // and it separates the two open planes joined by the corner fake bond
      g.colour[i] = (uint8_t)((cyc3(x, L, true) + cyc3(y, L, true) + cyc3(z, Lz, true)) % 3);
    }
    ok = proper(g);
  }
  if (!ok) {
    // greedy colouring in site order (degree 6: at most 7 colours)
    g.ncol = 0;
    for (int i = 0; i < V; ++i) {
      unsigned used = 0;
      for (int d = 0; d < 6; ++d) {
        const int p = g.nb[(size_t)i * 6 + d];
        if (p < i) used |= 1u << g.colour[p];
      }
      int c = 0;
      while (used >> c & 1) ++c;
      g.colour[i] = (uint8_t)c;
      g.ncol = std::max(g.ncol, c + 1);
    }
    if (!proper(g)) return false;
  }
  g.col_off.assign((size_t)g.ncol + 1, 0);
  for (int i = 0; i < V; ++i) ++g.col_off[g.colour[i] + 1];
  for (int c = 0; c < g.ncol; ++c) g.col_off[c + 1] += g.col_off[c];
  g.col_sites.assign((size_t)V, 0);
  std::vector<int32_t> fill(g.col_off.begin(), g.col_off.end() - 1);
  for (int i = 0; i < V; ++i) g.col_sites[fill[g.colour[i]]++] = i;
  // half-edge mates form an involution
  for (int h = 0; h < 6 * V; ++h)
    if (g.mate[g.mate[h]] != h || g.nb[g.mate[h]] != h / 6) return false;
  return true;
}

namespace {
inline uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// xoshiro256++ stream of word w of a job: state from splitmix64 of the seed
// offset by w.
ea_xoshiro word_stream(uint64_t seed, int w) {
  ea_xoshiro x;
  std::memset(&x, 0, sizeof(x));
  uint64_t sm = seed + (uint64_t)w * 0xD1B54A32D192ED03ULL;
  for (int k = 0; k < 4; ++k) x.s[k] = splitmix64(sm);
  return x;
}

// Runs f(w) for w = 0..n-1 on up to 16 host threads (each word has its own
// stream, so the order does not matter).
template <class F>
void for_words(int n, F f) {
  const int nth = std::max(1, std::min({n, 16, (int)std::thread::hardware_concurrency()}));
  if (nth == 1) {
    for (int w = 0; w < n; ++w) f(w);
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < nth; ++t)
    pool.emplace_back([=] {
      for (int w = t; w < n; w += nth) f(w);
    });
  for (auto &th : pool) th.join();
}
}  // namespace

// Couplings [w][site][slot]: every bit is one sample's +-J (bit 1 = the bond
// is unsatisfied when the two spins are equal).  Half-edges are visited in
// (site, slot) order; the first end of each bond draws its word, the other
// end copies it.
void sp_couplings(const SpGraph &g, int nwords, uint64_t seed_J, uint64_t *J) {
  for_words(nwords, [&g, seed_J, J](int w) {
    ea_xoshiro x = word_stream(seed_J, w);
    uint64_t *Jw = J + (size_t)w * g.V * 6;
    for (int h = 0; h < 6 * g.V; ++h) Jw[h] = g.mate[h] > h ? xo_next(x) : Jw[g.mate[h]];
  });
}

// Initial spins [w][site][rep][slot], one word per draw in that order.
void sp_spins(const SpGraph &g, int nwords, int NR, int NB, uint64_t seed_u, uint64_t *S) {
  const size_t per = (size_t)g.V * NR * NB;
  for_words(nwords, [per, seed_u, S](int w) {
    ea_xoshiro x = word_stream(seed_u, w);
    for (size_t i = 0; i < per; ++i) S[(size_t)w * per + i] = xo_next(x);
  });
}

}  // namespace eagb
