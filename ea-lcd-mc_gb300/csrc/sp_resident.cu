// sp_resident.cu -- resident bin kernel of small sample-packed jobs.
//
// A job too small to fill the GPU spends a per-phase launch on every colour
// pass, energy count, tempering step and permute, and each of those phases
// is a short latency-bound chain.  For bins without cluster moves, a job
// whose words fit in the shared memory of one thread-block cluster runs
// instead as three launches per chunk of sweeps:
//
//   k_sp_ctr_chain  the Philox counters of every colour pass of the chunk: one
//                   thread per replica steps its xoshiro256++ and
//                   Parisi-Rapuano generators (the counters never depend on
//                   the spins), the states staged in SMEM;
//   k_sp_draw       the three random words of every (pass, site, replica,
//                   slot) at once on the whole GPU -- the integer-heavy part
//                   of a sweep, now fully parallel;
//   k_sp_resident   one cluster of up to 16 CTAs holds the spin and coupling
//                   words in distributed shared memory (CTA c owns a run of
//                   sites) and runs every sweep, energy count, tempering
//                   step, permute and measurement of the chunk, phases
//                   separated by cluster barriers; neighbour words on other
//                   CTAs are read through DSMEM.
//
// Every phase computes what the per-phase kernels of sp.cu compute (same
// random words, update rule, bit-sliced counts, FP64 tempering rule and
// Philox uniforms, same order of the floating-point additions), so a job's
// words, energies, swaps and averages are identical either way.
#include <cooperative_groups.h>

#include <algorithm>

#include "kernels_dev.cuh"
#include "sp.cuh"

namespace cg = cooperative_groups;

namespace eagb {

constexpr int kResThreads = 512;
// bit planes of the per-sample counts summed over a warp: a CTA holds at most
// (2^15 - 1) / 6 sites
constexpr int kResPlanes = 15;
constexpr int kResMaxSites = ((1 << kResPlanes) - 1) / 6;

// ---------------------------------------------------------------------------
// Counters of npass consecutive colour passes (the fill step of sp.cu's
// k_sp_fill, repeated): pass p uses time counter iter0 + p and its parity.
// ---------------------------------------------------------------------------
__global__ void k_sp_ctr_chain(const __grid_constant__ SpDev d, int npass, uint4 *ctrs) {
  extern __shared__ __align__(16) unsigned char sm[];
  ea_hq *hs = reinterpret_cast<ea_hq *>(sm);
  ea_xoshiro *xs = reinterpret_cast<ea_xoshiro *>(hs + d.NR);
  const int NR = d.NR;
  const int nh = NR * (int)(sizeof(ea_hq) / 8), nx = NR * (int)(sizeof(ea_xoshiro) / 8);
  u64 *h64 = reinterpret_cast<u64 *>(hs), *x64 = reinterpret_cast<u64 *>(xs);
  const u64 *hg = reinterpret_cast<const u64 *>(d.prc), *xg = reinterpret_cast<const u64 *>(d.xo);
  for (int i = threadIdx.x; i < nh; i += blockDim.x) h64[i] = hg[i];
  for (int i = threadIdx.x; i < nx; i += blockDim.x) x64[i] = xg[i];
  const long long iter0 = *d.iter;
  __syncthreads();
  const int r = threadIdx.x;
  if (r < NR) {
    uint4 c = make_uint4(0u, 0u, 0u, 0u);
    for (int p = 0; p < npass; ++p) {
      const long long it = iter0 + p;
      c = next_counter(xs + r, hs + r, it, (int)(it & 1), d.jobid);
      ctrs[(size_t)p * NR + r] = c;
    }
    if (npass > 0) d.ctr[r] = c;
  }
  __syncthreads();
  u64 *hw = reinterpret_cast<u64 *>(d.prc), *xw = reinterpret_cast<u64 *>(d.xo);
  for (int i = threadIdx.x; i < nh; i += blockDim.x) hw[i] = h64[i];
  for (int i = threadIdx.x; i < nx; i += blockDim.x) xw[i] = x64[i];
  if (threadIdx.x == 0) *d.iter = iter0 + npass;
}

// ---------------------------------------------------------------------------
// Random words of nsweep sweeps: one thread per (sweep, colour, site of the
// colour, replica, slot), the words sp_pass_body draws for it (thresholds
// through the read-only cache).  Per sweep the colours follow each other;
// colour k's block holds 3 planes of NR * NB * n_k words, item (r, b, kk) at
// (r * NB + b) * n_k + kk of each plane (the site fastest, as the resident
// kernel's lanes read them).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sp_draw(const __grid_constant__ SpDev d, int nsweep, const uint4 *ctrs,
                                                 u64 *R) {
  const int NB = d.NB, NR = d.NR, G = NR * NB, V = d.V, ncol = d.ncol;
  const long long per = (long long)V * G;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= per * nsweep) return;
  const int s = (int)(t / per);
  const int rem = (int)(t - (long long)s * per);
  int k = 0;
  while (k + 1 < ncol && rem >= d.col_off[k + 1] * G) ++k;
  const int nk = d.col_off[k + 1] - d.col_off[k];
  const int e = rem - d.col_off[k] * G;
  const int col = e / nk, kk = e - col * nk, r = col / NB, b = col - r * NB;
  const int site = __ldg(d.col_sites + d.col_off[k] + kk);
  const uint4 c = ctrs[((size_t)s * ncol + k) * NR + r];
  const uint32_t tp = (uint32_t)(((size_t)b * V + site) * NR + r);
  const uint32_t key = __ldg(d.keys + r);
  const u64 *cum = d.cum + b * 256;
  const uint16_t *pre = d.pre + b * 256;
  uint32_t w[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) w[q] = rnd_word<true>(c.x + q, c.y, c.z + tp, c.w, key, tp, cum, pre);
  u64 *Rs = R + (size_t)s * 3 * per + (size_t)3 * d.col_off[k] * G;
  const size_t pl = (size_t)nk * G;
  Rs[e] = ((u64)w[0] << 32) | w[1];
  Rs[pl + e] = ((u64)w[2] << 32) | w[3];
  Rs[2 * pl + e] = ((u64)w[4] << 32) | w[5];
}

// ---------------------------------------------------------------------------
// Tempering uniforms of npt steps (sp_pt_body's draw): Philox4x32-10 of
// (step, pair, chain) keyed by the tempering seed, as FNORM * u in FP64 (an
// exact scaling of u rounded to 53 bits), stored as the double's bits.
// X: [step][word x replica][pair][sample].
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sp_pt_uniforms(const __grid_constant__ SpDev d, int npt, u64 *X) {
  const int NR = d.NR, NP = d.NB - 1, nunits = d.nw * NR;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)npt * nunits * NP * 64) return;
  const int lane = (int)(t & 63);
  long long rest = t >> 6;
  const int pi = (int)(rest % NP);
  rest /= NP;
  const int u = (int)(rest % nunits), j = (int)(rest / nunits);
  const int w = u / NR, r = u - w * NR;
  const unsigned long long step = *d.ptstep + (unsigned long long)j;
  const uint32_t chain = (uint32_t)(((size_t)w * 64 + lane) * NR + r);
  uint32_t v0 = (uint32_t)step, v1 = (uint32_t)(step >> 32), v2 = (uint32_t)pi, v3 = chain;
  philox10(v0, v1, v2, v3, (uint32_t)d.pt_seed, (uint32_t)(d.pt_seed >> 32));
  const double FNORM = 5.4210108624275218e-20;
  X[t] = (u64)__double_as_longlong(__dmul_rn(FNORM, __ull2double_rn(((u64)v0 << 32) | v1)));
}

// ---------------------------------------------------------------------------
// The resident kernel's phases.  Site i of the lattice lives in CTA i / nslm
// at local index i % nslm.  SMEM arrays keep the site (or the sample) as the
// fastest index, so that the lanes of a warp -- consecutive sites of one
// (replica, slot) column, or consecutive samples of one chain -- touch
// consecutive words:
//   S   [nw][NR*NB][nslm]  spin words         J    [nw][6][nslm] coupling words
//   nbl [6][nslm]          neighbour of each bond slot as (CTA << 16 | local index)
//   lst [nsl]              the CTA's sites, colour by colour
// and per chain (unit u = (word, replica) = lu * ncta + rank, 64 samples):
//   U2s, Es, Av, Ps [upc][NB][64]    As [upc][NB-1][64]    Ms [upc][NB-1]
// ---------------------------------------------------------------------------
struct ResCta {
  int rank, site_lo, nsl;
};

struct ResShared {
  u64 *S, *J;
  u64 *Ms;       // lanes that swapped, per pair
  u64 *Mall;     // [nunits][NB-1] every chain's masks, gathered for the permute
  long long *Av; // the bin's energy sums (integers: exactly the double sums, all below 2^53)
  u64 *Tab;      // [ntab] host-libm exp table as bits (when staged)
  int32_t *U2s;  // counts of the whole lattice (DSMEM atomics of every CTA)
  int32_t *Es;
  uint32_t *As;
  uint32_t *nbl;
  int32_t *EO;   // [NB] exp table offsets
  int32_t *SG;   // [NB-1] sign of -(beta[i+1] - beta[i])
  uint16_t *lst;
  uint8_t *Ps;
  u64 *Xs;       // [upc][NB-1][64] tempering uniforms of the step
};

__host__ __device__ inline size_t res_smem_bytes(int nw, int nslm, int NR, int NB, int upc, int ntab) {
  const size_t G = (size_t)NR * NB, NP = NB - 1, nunits = (size_t)nw * NR, U = (size_t)upc * 64;
  const size_t b = 8 * ((size_t)nw * nslm * G + (size_t)nw * nslm * 6 + upc * NP + nunits * NP + U * NB + (size_t)ntab +
                        U * NP) +
                   4 * (2 * U * NB + U * NP + (size_t)nslm * 6 + NB + NP) + 2 * (size_t)nslm + U * NB;
  return (b + 15) & ~(size_t)15;
}

__device__ __forceinline__ ResShared res_carve(unsigned char *smem, const SpResDev &p) {
  const SpDev &d = p.d;
  const size_t G = (size_t)d.NR * d.NB, NP = d.NB - 1, nunits = (size_t)d.nw * d.NR, U = (size_t)p.upc * 64;
  ResShared s;
  s.S = reinterpret_cast<u64 *>(smem);
  s.J = s.S + (size_t)d.nw * p.nslm * G;
  s.Ms = s.J + (size_t)d.nw * p.nslm * 6;
  s.Mall = s.Ms + (size_t)p.upc * NP;
  s.Xs = s.Mall + nunits * NP;
  s.Av = reinterpret_cast<long long *>(s.Xs + U * NP);
  s.Tab = reinterpret_cast<u64 *>(s.Av + U * d.NB);
  s.U2s = reinterpret_cast<int32_t *>(s.Tab + p.ntab);
  s.Es = s.U2s + U * d.NB;
  s.As = reinterpret_cast<uint32_t *>(s.Es + U * d.NB);
  s.nbl = s.As + U * NP;
  s.EO = reinterpret_cast<int32_t *>(s.nbl + (size_t)p.nslm * 6);
  s.SG = s.EO + d.NB;
  s.lst = reinterpret_cast<uint16_t *>(s.SG + NP);
  s.Ps = reinterpret_cast<uint8_t *>(s.lst + p.nslm);
  return s;
}

// The word of column Sc (this CTA's copy of a (word, column) row of S) at the
// site packed in nb, from this CTA or another one of the cluster.
__device__ __forceinline__ u64 res_word(const cg::cluster_group &cl, const ResCta &me, u64 *Sc, uint32_t nb) {
  const int own = (int)(nb >> 16), nl = (int)(nb & 0xFFFFu);
  return own == me.rank ? Sc[nl] : cl.map_shared_rank(Sc, own)[nl];
}

// One colour pass over the CTA's sites of colour k (sp_pass_body's update):
// a group of lpc lanes per (word, column), lanes over the colour's sites.
__device__ __forceinline__ void res_pass(const SpResDev &p, const cg::cluster_group &cl, const ResCta &me,
                                         const ResShared &s, int sweep, int k) {
  const SpDev &d = p.d;
  const int G = d.NR * d.NB, nslm = p.nslm;
  const int off = d.col_off[k], nk = d.col_off[k + 1] - off;
  const int kb = p.kr[me.rank][k], nkc = p.kr[me.rank + 1][k] - kb;
  if (nkc <= 0) return;
  int loff = 0;
  for (int c = 0; c < k; ++c) loff += p.kr[me.rank + 1][c] - p.kr[me.rank][c];
  const u64 *Rk = p.R + (size_t)sweep * 3 * d.V * G + (size_t)3 * off * G + kb;
  const size_t pl = (size_t)nk * G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int lpc = p.lpc_count, cpw = 32 / lpc, gl = lane & (lpc - 1), ncols = d.nw * G;
  for (int c = warp * cpw + lane / lpc; c < ncols; c += nwarp * cpw) {
    const int w = c / G, col = c - w * G;
    u64 *Sc = s.S + (size_t)c * nslm;
    const u64 *Jw = s.J + (size_t)w * 6 * nslm;
    const u64 *Rc = Rk + (size_t)col * nk;
    for (int kl = gl; kl < nkc; kl += lpc) {
      const int local = s.lst[loff + kl];
      const u64 r0 = __ldg(Rc + kl), r1 = __ldg(Rc + pl + kl), r2 = __ldg(Rc + 2 * pl + kl);
      const u64 sv = Sc[local];
      u64 f[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) f[q] = sv ^ Jw[(size_t)q * nslm + local] ^ res_word(cl, me, Sc, s.nbl[q * nslm + local]);
      Sc[local] = sv ^ flip_mask(f, r0, r1, r2);
    }
  }
}

// Asynchronous 8-byte global-to-SMEM copies (cp.async); a thread waits for
// all of its copies with cp_async_wait_all (a hardware wait) before the
// barrier that publishes them.
__device__ __forceinline__ void cp_async8(void *smem, const void *g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Tempering uniforms of this CTA's chains for step ptj into Xs.
__device__ __forceinline__ void res_stage_x(const SpResDev &p, const ResCta &me, const ResShared &s, int ptj) {
  const int NP = p.d.NB - 1, nunits = p.d.nw * p.d.NR, per = NP * 64;
  for (int t = threadIdx.x; t < p.upc * per; t += blockDim.x) {
    const int lu = t / per, e = t - lu * per, u = lu * p.ncta + me.rank;
    if (u < nunits) cp_async8(s.Xs + t, p.X + ((size_t)ptj * nunits + u) * per + e);
  }
  cp_async_commit();
}

__device__ __forceinline__ void res_count_add(u64 *P, int npl, const u64 f[6]) {
  const u64 x1 = f[0] ^ f[1] ^ f[2], y1 = (f[0] & f[1]) | (f[2] & (f[0] ^ f[1]));
  const u64 x2 = f[3] ^ f[4] ^ f[5], y2 = (f[3] & f[4]) | (f[5] & (f[3] ^ f[4]));
  const u64 z0 = x1 ^ x2, c0 = x1 & x2;
  const u64 z1 = y1 ^ y2 ^ c0, z2 = (y1 & y2) | (c0 & (y1 ^ y2));
  u64 cy = P[0] & z0;
  P[0] ^= z0;
  u64 t = P[1] ^ z1 ^ cy;
  cy = (P[1] & z1) | (cy & (P[1] ^ z1));
  P[1] = t;
  t = P[2] ^ z2 ^ cy;
  cy = (P[2] & z2) | (cy & (P[2] ^ z2));
  P[2] = t;
#pragma unroll
  for (int q = 3; q < npl; ++q) {
    const u64 h = P[q] & cy;
    P[q] ^= cy;
    cy = h;
  }
}

// A group of lpc lanes (8, 16 or 32; one (word, column) per group, lpc | 32)
// sums its bit-sliced counters (a butterfly of bit-sliced additions inside
// the group); then lane l of the group holds samples l, l + lpc, ... of the
// sum and adds them, times `scale`, to the counts of the chain (word,
// replica r) at slot b in the CTA that owns the chain (DSMEM atomics).
// Every lane of the warp takes part in the shuffles; `valid` lanes add.
template <int NPL>
__device__ __forceinline__ void res_count_flush(const SpResDev &p, const cg::cluster_group &cl, const ResCta &me,
                                                const ResShared &s, u64 *P, int lpc, bool valid, int w, int r, int b,
                                                int scale) {
  const int gl = threadIdx.x & (lpc - 1), NB = p.d.NB;
  for (int m = lpc >> 1; m >= 1; m >>= 1) {
    u64 cy = 0;
#pragma unroll
    for (int q = 0; q < NPL; ++q) {
      const u64 o = __shfl_xor_sync(0xffffffffu, P[q], m);
      const u64 t = P[q] ^ o ^ cy;
      cy = (P[q] & o) | (cy & (P[q] ^ o));
      P[q] = t;
    }
  }
  if (!valid) return;
  const int u = w * p.d.NR + r, own = u % p.ncta, lu = u / p.ncta;
  int32_t *dst = (own == me.rank ? s.U2s : cl.map_shared_rank(s.U2s, own)) + ((size_t)lu * NB + b) * 64;
  for (int smp = gl; smp < 64; smp += lpc) {
    int c = 0;
#pragma unroll
    for (int q = 0; q < NPL; ++q) c |= (int)((P[q] >> smp) & 1ull) << q;
    atomicAdd(dst + smp, scale * c);
  }
}

// The last colour pass of a sweep on a two-colour lattice with the energy
// counted on the way (sp.cu's update, then sp_energy_body's count): every bond
// joins a colour-0 site to a colour-1 site and both ends hold its coupling,
// so U2 is twice the unsatisfied half-edges of the colour-1 sites, all final
// once their pass has flipped them (f ^= flip).  A warp per (word, column),
// lanes over the colour's sites.
template <int NPL>
__device__ __forceinline__ void res_pass_count(const SpResDev &p, const cg::cluster_group &cl, const ResCta &me,
                                               const ResShared &s, int sweep, int k) {
  const SpDev &d = p.d;
  const int NB = d.NB, G = d.NR * NB, nslm = p.nslm;
  const int off = d.col_off[k], nk = d.col_off[k + 1] - off;
  const int kb = p.kr[me.rank][k], nkc = p.kr[me.rank + 1][k] - kb;
  int loff = 0;
  for (int c = 0; c < k; ++c) loff += p.kr[me.rank + 1][c] - p.kr[me.rank][c];
  const u64 *Rk = p.R + (size_t)sweep * 3 * d.V * G + (size_t)3 * off * G + kb;
  const size_t pl = (size_t)nk * G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int lpc = p.lpc_count, cpw = 32 / lpc, gl = lane & (lpc - 1), ncols = d.nw * G;
  for (int base = warp * cpw; base < ncols; base += nwarp * cpw) {
    const int c = base + lane / lpc;
    const bool valid = c < ncols;
    const int cc = valid ? c : 0, w = cc / G, col = cc - w * G, r = col / NB, b = col - r * NB;
    u64 *Sc = s.S + (size_t)cc * nslm;
    const u64 *Jw = s.J + (size_t)w * 6 * nslm;
    const u64 *Rc = Rk + (size_t)col * nk;
    u64 P[NPL];
#pragma unroll
    for (int q = 0; q < NPL; ++q) P[q] = 0;
    for (int kl = gl; valid && kl < nkc; kl += lpc) {
      const int local = s.lst[loff + kl];
      const u64 r0 = __ldg(Rc + kl), r1 = __ldg(Rc + pl + kl), r2 = __ldg(Rc + 2 * pl + kl);
      const u64 sv = Sc[local];
      u64 f[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) f[q] = sv ^ Jw[(size_t)q * nslm + local] ^ res_word(cl, me, Sc, s.nbl[q * nslm + local]);
      const u64 m = flip_mask(f, r0, r1, r2);
      Sc[local] = sv ^ m;
#pragma unroll
      for (int q = 0; q < 6; ++q) f[q] ^= m;
      res_count_add(P, NPL, f);
    }
    res_count_flush<NPL>(p, cl, me, s, P, lpc, valid, w, r, b, 2);
  }
}

// Unsatisfied half-edges per (word, sample, replica, slot) (sp_energy_body's
// count): a warp per (word, column) of the CTA, lanes over its sites,
// bit-sliced counters summed over the warp by a butterfly of bit-sliced
// additions; lane l then holds samples l and l + 32 and adds them to the
// chain's counts in the CTA that owns the chain (DSMEM atomics).
template <int NPL>
__device__ __forceinline__ void res_energy(const SpResDev &p, const cg::cluster_group &cl, const ResCta &me,
                                           const ResShared &s) {
  const SpDev &d = p.d;
  const int NB = d.NB, G = d.NR * NB, nslm = p.nslm;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int lpc = p.lpc_energy, cpw = 32 / lpc, gl = lane & (lpc - 1), ncols = d.nw * G;
  for (int base = warp * cpw; base < ncols; base += nwarp * cpw) {
    const int c = base + lane / lpc;
    const bool valid = c < ncols;
    const int cc = valid ? c : 0, w = cc / G, col = cc - w * G, r = col / NB, b = col - r * NB;
    u64 *Sc = s.S + (size_t)cc * nslm;
    const u64 *Jw = s.J + (size_t)w * 6 * nslm;
    u64 P[NPL];
#pragma unroll
    for (int q = 0; q < NPL; ++q) P[q] = 0;
    for (int i = gl; valid && i < me.nsl; i += lpc) {
      const u64 sv = Sc[i];
      u64 f[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) f[q] = sv ^ Jw[(size_t)q * nslm + i] ^ res_word(cl, me, Sc, s.nbl[q * nslm + i]);
      res_count_add(P, NPL, f);
    }
    res_count_flush<NPL>(p, cl, me, s, P, lpc, valid, w, r, b, 1);
  }
}

// One tempering step of the CTA's chains (sp_pt_body's rule and uniforms).
// pt = -(beta[i+1] - beta[i]) * dE is >= 0 exactly when dE has the sign of
// -(beta[i+1] - beta[i]) (or that factor is zero), so the walk needs no FP64:
// FNORM * u is formed beforehand for every pair, and both it and the table's
// exp values are non-negative doubles, which order as their bit patterns.
// With `measure`, the slots' energies are added to the bin's sums
// (sp_measure_u2_body after a tempering step).  The chains' counts are then
// cleared for the next energy phase.
__device__ __forceinline__ void res_tempering(const SpResDev &p, const ResCta &me, const ResShared &s, int ptj,
                                              bool measure, bool last) {
  const SpDev &d = p.d;
  const int NB = d.NB, NR = d.NR, G = NR * NB, NP = NB - 1, nunits = d.nw * NR, upc = p.upc, ncta = p.ncta;
  const int nt = 3 * d.V;
  for (int lu = threadIdx.x >> 6; lu < upc; lu += blockDim.x >> 6) {
    const int u = lu * ncta + me.rank;
    if (u >= nunits) continue;  // the same for the unit's 64 threads
    const int lane = threadIdx.x & 63;
    int32_t *Eo = s.Es + (size_t)lu * NB * 64 + lane;
    uint8_t *Po = s.Ps + (size_t)lu * NB * 64 + lane;
    const int32_t *Uo = s.U2s + (size_t)lu * NB * 64 + lane;
    const u64 *xo = s.Xs + (size_t)lu * NP * 64 + lane;
    uint32_t *ao = s.As + (size_t)lu * NP * 64 + lane;
    uint32_t *Mh = reinterpret_cast<uint32_t *>(s.Ms + (size_t)lu * NP);
    // the pairs in chunks of 4: every input that does not depend on the
    // carried configuration is read first, then the 4 decisions are taken
    // in order (the table entry is read whether or not it decides: index 0
    // when m is out of range; the table has at least one entry)
    int carry_e = nt - Uo[0];
    uint32_t carry_p = Po[0];
    for (int i0 = 0; i0 < NP; i0 += 4) {
      int e1[4], sg[4], eb[4], nx[4];
      uint32_t p1[4];
      u64 x[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int i = min(i0 + j, NP - 1);
        e1[j] = nt - Uo[(i + 1) * 64];
        p1[j] = Po[(i + 1) * 64];
        x[j] = xo[(size_t)i * 64];
        sg[j] = s.SG[i];
        eb[j] = s.EO[i];
        nx[j] = s.EO[i + 1] - eb[j];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int i = i0 + j;
        if (i >= NP) break;
        const int dE = e1[j] - carry_e, m = (-dE) >> 1;
        const bool up = sg[j] == 0 || (sg[j] > 0 ? dE >= 0 : dE <= 0);
        const bool inr = m >= 1 && m <= nx[j];
        const int ti = inr ? eb[j] + m - 1 : 0;
        const u64 tv = p.ntab ? s.Tab[ti] : (u64)__double_as_longlong(__ldg(d.exptab + ti));
        const bool change = up || (inr ? x[j] < tv : x[j] == 0);
        Eo[i * 64] = change ? e1[j] : carry_e;
        Po[i * 64] = (uint8_t)(change ? p1[j] : carry_p);
        ao[i * 64] += change ? 1u : 0u;
        carry_e = change ? carry_e : e1[j];
        carry_p = change ? carry_p : p1[j];
        Mh[2 * i + (lane >> 5)] = __ballot_sync(0xffffffffu, change);
      }
    }
    Eo[NP * 64] = carry_e;
    Po[NP * 64] = (uint8_t)carry_p;
    if (measure) {
      long long *av = s.Av + (size_t)lu * NB * 64 + lane;
      for (int b = 0; b < NB; ++b) av[b * 64] += Eo[b * 64];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < upc * 64 * NB; i += blockDim.x) {
    if (last) {
      const int lane = i & 63, rest = i >> 6, lu = rest / NB, b = rest - lu * NB;
      const int u = lu * ncta + me.rank;
      if (u < nunits) {
        const int w = u / NR, r = u - w * NR;
        d.U2[((size_t)w * 64 + lane) * G + (size_t)r * NB + b] = s.U2s[i];
      }
    }
    s.U2s[i] = 0;
  }
}

// The accepted swaps applied to the CTA's rows (sp_permute_body), the masks
// of every chain gathered from their CTAs first; rows (word, replica, site)
// with the site fastest.
__device__ __forceinline__ void res_permute(const SpResDev &p, const cg::cluster_group &cl, const ResCta &me,
                                            const ResShared &s) {
  const SpDev &d = p.d;
  const int NB = d.NB, NR = d.NR, NP = NB - 1, nunits = d.nw * NR, ncta = p.ncta, nslm = p.nslm;
  for (int i = threadIdx.x; i < nunits * NP; i += blockDim.x) {
    const int u = i / NP, pi = i - u * NP, own = u % ncta;
    const size_t o = (size_t)(u / ncta) * NP + pi;
    s.Mall[i] = own == me.rank ? s.Ms[o] : cl.map_shared_rank(s.Ms, own)[o];
  }
  __syncthreads();
  const int rows = nunits * me.nsl;
  for (int t = threadIdx.x; t < rows; t += blockDim.x) {
    const int u = t / me.nsl, i = t - u * me.nsl;  // u = w * NR + r
    u64 *row = s.S + (size_t)u * NB * nslm + i;    // column r * NB + b of word w
    const u64 *M = s.Mall + (size_t)u * NP;
    u64 cur = row[0];
    for (int b = 0; b < NP; ++b) {
      const u64 m = M[b], nxt = row[(size_t)(b + 1) * nslm], x = (cur ^ nxt) & m;
      row[(size_t)b * nslm] = cur ^ x;
      cur = nxt ^ x;
    }
    row[(size_t)NP * nslm] = cur;
  }
}

// NPL: bit planes of a warp's per-sample count, 6 * nslm < 2^NPL.
template <int NPL>
__global__ void __launch_bounds__(kResThreads, 1) k_sp_resident(const __grid_constant__ SpResDev p) {
  const cg::cluster_group cl = cg::this_cluster();
  const SpDev &d = p.d;
  const int NB = d.NB, NR = d.NR, G = NR * NB, NP = NB - 1, V = d.V, nw = d.nw, ncol = d.ncol;
  const int nslm = p.nslm, ncta = p.ncta, upc = p.upc, nunits = nw * NR;
  ResCta me;
  me.rank = (int)cl.block_rank();
  me.site_lo = me.rank * nslm;
  me.nsl = min(nslm, V - me.site_lo);
  extern __shared__ __align__(16) unsigned char smem[];
  const ResShared s = res_carve(smem, p);
  const int tid = threadIdx.x, nth = blockDim.x;

  // the CTA's words and neighbour table, its sites by colour, the tempering
  // tables, and the energies, slot ids, acceptances and sums of its chains
  // (global memory reads in global order, SMEM writes transposed)
  const int nS = nw * me.nsl * G, nJ = nw * me.nsl * 6;
  for (int i = tid; i < nS; i += nth) {
    const int col = i % G, rest = i / G, si = rest % me.nsl, w = rest / me.nsl;
    s.S[((size_t)w * G + col) * nslm + si] = d.S[((size_t)w * V + me.site_lo + si) * G + col];
  }
  for (int i = tid; i < nJ; i += nth) {
    const int q = i % 6, rest = i / 6, si = rest % me.nsl, w = rest / me.nsl;
    s.J[((size_t)w * 6 + q) * nslm + si] = d.J[((size_t)w * V + me.site_lo + si) * 6 + q];
  }
  for (int i = tid; i < me.nsl * 6; i += nth) {
    const int nbs = __ldg(d.nb + (size_t)me.site_lo * 6 + i), own = nbs / nslm, q = i % 6, si = i / 6;
    s.nbl[q * nslm + si] = ((uint32_t)own << 16) | (uint32_t)(nbs - own * nslm);
  }
  for (int k = 0, loff = 0; k < ncol; ++k) {
    const int kb = p.kr[me.rank][k], nkc = p.kr[me.rank + 1][k] - kb, off = d.col_off[k];
    for (int j = tid; j < nkc; j += nth) s.lst[loff + j] = (uint16_t)(__ldg(d.col_sites + off + kb + j) - me.site_lo);
    loff += nkc;
  }
  for (int i = tid; i < NB; i += nth) s.EO[i] = d.expoff[i];
  for (int i = tid; i < NP; i += nth) {
    const double f = -__dsub_rn(d.betas[i + 1], d.betas[i]);
    s.SG[i] = f > 0.0 ? 1 : (f < 0.0 ? -1 : 0);
  }
  for (int i = tid; i < p.ntab; i += nth) s.Tab[i] = (u64)__double_as_longlong(d.exptab[i]);
  for (int i = tid; i < upc * 64 * NB; i += nth) {
    s.U2s[i] = 0;
    const int lane = i & 63, rest = i >> 6, lu = rest / NB, b = rest - lu * NB;
    const int u = lu * ncta + me.rank;
    if (u >= nunits) continue;
    const int w = u / NR, r = u - w * NR;
    const size_t o = ((size_t)w * 64 + lane) * G + (size_t)r * NB + b;
    s.Es[i] = d.E[o];
    s.Ps[i] = d.perm[o];
    s.Av[i] = (long long)d.avgE[o];
  }
  for (int i = tid; i < upc * 64 * NP; i += nth) {
    const int lane = i & 63, rest = i >> 6, lu = rest / NP, pi = rest - lu * NP;
    const int u = lu * ncta + me.rank;
    if (u >= nunits) continue;
    const int w = u / NR, r = u - w * NR;
    s.As[i] = d.acc[(((size_t)w * 64 + lane) * NR + r) * NP + pi];
  }
  const unsigned long long step0 = *d.ptstep;
  cl.sync();

  int sweep = 0, ptj = 0;
  for (int it = 0; it < p.nit; ++it)
    for (int im = 0; im < p.mesfr; ++im)
      for (int ih = 0; ih < p.houfr; ++ih) {
        res_stage_x(p, me, s, ptj);
        for (int sw = 0; sw < p.ptfr; ++sw, ++sweep)
          for (int k = 0; k < ncol; ++k) {
            if (p.pair_energy && k == ncol - 1 && sw == p.ptfr - 1) res_pass_count<NPL>(p, cl, me, s, sweep, k);
            else res_pass(p, cl, me, s, sweep, k);
            cp_async_wait_all();  // this step's uniforms (staged before the first pass)
            cl.sync();
          }
        if (!p.pair_energy) {
          res_energy<NPL>(p, cl, me, s);
          cl.sync();
        }
        const bool lastpt = im == p.mesfr - 1 && ih == p.houfr - 1;
        res_tempering(p, me, s, ptj, p.measure && lastpt, lastpt && it == p.nit - 1);
        cl.sync();
        res_permute(p, cl, me, s);
        cl.sync();
        ++ptj;
      }

  // back to global memory
  for (int i = tid; i < nS; i += nth) {
    const int col = i % G, rest = i / G, si = rest % me.nsl, w = rest / me.nsl;
    d.S[((size_t)w * V + me.site_lo + si) * G + col] = s.S[((size_t)w * G + col) * nslm + si];
  }
  for (int i = tid; i < upc * 64 * NB; i += nth) {
    const int lane = i & 63, rest = i >> 6, lu = rest / NB, b = rest - lu * NB;
    const int u = lu * ncta + me.rank;
    if (u >= nunits) continue;
    const int w = u / NR, r = u - w * NR;
    const size_t o = ((size_t)w * 64 + lane) * G + (size_t)r * NB + b;
    d.E[o] = s.Es[i];
    d.perm[o] = s.Ps[i];
    d.avgE[o] = (double)s.Av[i];
  }
  for (int i = tid; i < upc * 64 * NP; i += nth) {
    const int lane = i & 63, rest = i >> 6, lu = rest / NP, pi = rest - lu * NP;
    const int u = lu * ncta + me.rank;
    if (u >= nunits) continue;
    const int w = u / NR, r = u - w * NR;
    d.acc[(((size_t)w * 64 + lane) * NR + r) * NP + pi] = s.As[i];
  }
  for (int i = tid; i < upc * NP; i += nth) {
    const int lu = i / NP, pi = i - lu * NP, u = lu * ncta + me.rank;
    if (u < nunits) d.M[(size_t)u * NP + pi] = s.Ms[i];
  }
  if (me.rank == 0 && tid == 0) *d.ptstep = step0 + (unsigned long long)ptj;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int res_lanes(int sites) { return sites <= 32 ? 8 : sites <= 96 ? 16 : 32; }

// Counter planes of the energy phase's warp sums: 6 * nslm < 2^NPL.
static int res_npl(int nslm) { return 6 * nslm < (1 << 10) ? 10 : kResPlanes; }

template <int NPL>
static cudaError_t res_attrs() {
  cudaError_t e = cudaFuncSetAttribute(k_sp_resident<NPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sp_resident<NPL>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

cudaError_t sp_res_setup() {
  cudaError_t e = res_attrs<10>();
  if (e == cudaSuccess) e = res_attrs<kResPlanes>();
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_sp_ctr_chain, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             64 * (int)(sizeof(ea_hq) + sizeof(ea_xoshiro)));
  return e;
}

static cudaLaunchConfig_t res_config(int ncta, size_t smem, cudaStream_t st, cudaLaunchAttribute *at) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)ncta);
  cfg.blockDim = dim3(kResThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  at->id = cudaLaunchAttributeClusterDimension;
  at->val.clusterDim.x = (unsigned)ncta;
  at->val.clusterDim.y = 1;
  at->val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

// Whether the job's share of the widest split (sites split evenly over 16
// CTAs) fits one CTA's shared memory (the exp table left in global memory).
bool sp_res_fits(int L, int Lz, int nw, int NR, int NB) {
  if (NB < 2 || L < 1 || Lz < 1) return false;
  const long long V = (long long)L * L * Lz, nslm = (V + kResMaxCta - 1) / kResMaxCta;
  const int ncta = (int)((V + nslm - 1) / nslm);
  if (nslm > kResMaxSites) return false;
  const int upc = (nw * NR + ncta - 1) / ncta;
  return res_smem_bytes(nw, (int)nslm, NR, NB, upc, 0) <= 227 * 1024;
}

// The most CTAs (sites split into equal runs, at most 16) whose cluster the
// GPU can hold with the job's shared memory; none when a CTA's share does
// not fit.  The exp table is staged in SMEM when it fits beside the words.
bool sp_res_plan(const SpDev &d, const int32_t *col_sites, int ntab, SpResPlan &pl) {
  if (d.ncol < 1 || d.ncol > kResMaxColours || d.NB < 2) return false;
  const int nunits = d.nw * d.NR;
  const size_t lim = 227 * 1024;
  int last = 0;
  for (int want = std::min(kResMaxCta, d.V); want >= 1; --want) {
    const int nslm = (d.V + want - 1) / want, ncta = (d.V + nslm - 1) / nslm;
    if (ncta == last) continue;
    last = ncta;
    if (nslm > kResMaxSites) return false;
    const int upc = (nunits + ncta - 1) / ncta;
    int nt = ntab;
    size_t smem = res_smem_bytes(d.nw, nslm, d.NR, d.NB, upc, nt);
    if (smem > lim) smem = res_smem_bytes(d.nw, nslm, d.NR, d.NB, upc, nt = 0);
    if (smem > lim) return false;
    const int npl = res_npl(nslm);
    cudaLaunchAttribute at;
    const cudaLaunchConfig_t cfg = res_config(ncta, smem, nullptr, &at);
    int nclusters = 0;
    const cudaError_t e = npl == 10 ? cudaOccupancyMaxActiveClusters(&nclusters, k_sp_resident<10>, &cfg)
                                    : cudaOccupancyMaxActiveClusters(&nclusters, k_sp_resident<kResPlanes>, &cfg);
    if (e != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (nclusters < 1) continue;
    for (int c = 0; c <= ncta; ++c)
      for (int k = 0; k < d.ncol; ++k) {
        const int32_t *b = col_sites + d.col_off[k], *e2 = col_sites + d.col_off[k + 1];
        pl.kr[c][k] = (int)(std::lower_bound(b, e2, c * nslm) - b);
      }
    pl.ncta = ncta;
    pl.nslm = nslm;
    pl.upc = upc;
    // lanes per counted column: about 2-4 sites a lane (a butterfly level
    // costs the same whatever the number of sites behind it)
    int most = 0;
    for (int c = 0; c < ncta; ++c) most = std::max(most, pl.kr[c + 1][d.ncol - 1] - pl.kr[c][d.ncol - 1]);
    pl.lpc_count = res_lanes(most);
    pl.lpc_energy = res_lanes(nslm);
    pl.ntab = nt;
    pl.npl = npl;
    pl.smem = smem;
    return true;
  }
  return false;
}

size_t sp_res_launch_sweeps(size_t V, size_t G, const ea_cadence *cad) {
  const size_t spi = (size_t)cad->mesfr * cad->houfr * cad->ptfr, bytes_sweep = 24 * V * G;
  if (cad->cluster) {
    // one launch per block of houfr x ptfr sweeps between two cluster moves
    const size_t blk = (size_t)cad->houfr * cad->ptfr;
    return blk >= (size_t)kResMinBlock && blk * bytes_sweep <= ((size_t)256 << 20) ? blk : 0;
  }
  if (spi * bytes_sweep > ((size_t)256 << 20)) return 0;
  const size_t its = std::max<size_t>(1, ((size_t)16 << 20) / (bytes_sweep * spi));
  return std::min(its, (size_t)std::max(cad->itmax, 1)) * spi;
}

cudaError_t sp_res_chunk(const SpResDev &p, const SpResPlan &pl, int npass, uint4 *ctrs, cudaStream_t st) {
  const SpDev &d = p.d;
  k_sp_ctr_chain<<<1, d.NR <= 32 ? 32 : 64, (size_t)d.NR * (sizeof(ea_hq) + sizeof(ea_xoshiro)), st>>>(d, npass, ctrs);
  const int nsweep = npass / d.ncol;
  const long long n = (long long)nsweep * d.V * d.NR * d.NB;
  k_sp_draw<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d, nsweep, ctrs, const_cast<u64 *>(p.R));
  const int npt = p.nit * p.mesfr * p.houfr;
  const long long nx = (long long)npt * d.nw * d.NR * (d.NB - 1) * 64;
  if (nx > 0) k_sp_pt_uniforms<<<(unsigned)((nx + 255) / 256), 256, 0, st>>>(d, npt, const_cast<u64 *>(p.X));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute at;
  const cudaLaunchConfig_t cfg = res_config(pl.ncta, pl.smem, st, &at);
  return pl.npl == 10 ? cudaLaunchKernelEx(&cfg, k_sp_resident<10>, p)
                      : cudaLaunchKernelEx(&cfg, k_sp_resident<kResPlanes>, p);
}

}  // namespace eagb
