// host.hpp -- host-side pieces of the job set-up (generators, geometry, packing).
// These run once per job on the CPU, as they do in the reference; the sweep,
// energy, tempering and cluster kernels run on the GPU (kernels.cu).
#pragma once
#include <cstdint>
#include <vector>
#include "eagb.h"

namespace eagb {

constexpr uint64_t kLcg = 3202034522624059733ULL;

// Parisi-Rapuano + LCG step (random_generator.h:62-67).
inline uint64_t hq_next(ea_hq &u) {
  u.ira[u.ip] = u.ira[u.ip1] + u.ira[u.ip2];
  u.PR = u.ira[u.ip] ^ u.ira[u.ip3];
  u.zseed = u.zseed * kLcg + 1;
  u.final = u.zseed + u.PR;
  ++u.ip; ++u.ip1; ++u.ip2; ++u.ip3;
  return u.final;
}

inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

// xoshiro256++ step (random_generator.h:50-59).
inline uint64_t xo_next(ea_xoshiro &u) {
  u.final = rotl64(u.s[0] + u.s[3], 23) + u.s[0];
  u.t = u.s[1] << 17;
  u.s[2] ^= u.s[0];
  u.s[3] ^= u.s[1];
  u.s[1] ^= u.s[2];
  u.s[0] ^= u.s[3];
  u.s[2] ^= u.t;
  u.s[3] = rotl64(u.s[3], 45);
  return u.final;
}

void hq_seed(ea_hq &u, uint64_t seed);
void seeds_from_one(uint64_t seed, uint64_t *out, int n);
void init_generators(uint64_t seed, ea_hq &prc, ea_xoshiro &xo, uint32_t &key);

// Derived sizes of the multispin geometry (header.h:50-66).
struct Geometry {
  int L = 0, Lz = 0, NB = 0, NR = 0, ns = 0, bc = 0;
  int msc_l = 0, msc_lz = 0, msc_s = 0, msc_v = 0, half = 0, V = 0;
  bool set(const ea_geom &g);
  size_t words_per_clone() const { return (size_t)half * NR; }
  size_t words_per_parity() const { return words_per_clone() * NB; }
  size_t words_per_sample() const { return 2 * words_per_parity(); }
};

// Neighbour half-site indices [parity][dir][half] and per-site flags
// [parity][half]: bits 0-5 rotate dir d, bit 6 top MSC plane, bit 7 bottom plane.
void neighbour_tables(const Geometry &g, std::vector<int32_t> &idx, std::vector<uint8_t> &flags);

void init_spin_bytes(const Geometry &g, uint64_t seed_u, std::vector<uint8_t> &uu);  // [NR][NB][V]
void pack_clone(const Geometry &g, const uint8_t *u, int rep, int clone, uint64_t *even, uint64_t *odd);
void unpack_clone(const Geometry &g, const uint64_t *even, const uint64_t *odd, int rep, int clone, uint8_t *u);
int init_couplings(const Geometry &g, uint64_t seed_J, uint8_t *J6);
void pack_couplings(const Geometry &g, const uint8_t *J6, uint64_t *Jw);
int scalar_energy(const Geometry &g, const uint8_t *u, const uint8_t *J6);

// 8-bit pre-search of the cumulative thresholds: entry b = (lo, hi) bounds of the
// byte drawn for any R whose top 8 bits are b.
void presearch8(const uint64_t *cum, uint16_t *pre);
constexpr int kPre11Stride = 2064;  // 2049 entries a temperature, padded to 16 bytes
void presearch11(const uint64_t *cum, uint8_t *pre);

// glibc exp() of every parallel-tempering exponent that can change a decision,
// laid out per beta pair: offsets[i] .. offsets[i+1] hold exp(pt) for
// dE = -2, -4, ... (pt = -(b[i+1]-b[i]) * dE).  Beyond a pair's range exp(pt) < 2^-72.
void pt_exp_table(const double *betas, int NB, std::vector<double> &vals, std::vector<int32_t> &offsets);

}  // namespace eagb
