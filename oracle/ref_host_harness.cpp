// ref_host_harness.cpp -- TEST INFRASTRUCTURE.
//
// Links the reference's own host code (PROGRAM/src/random_generator.cu,
// ini.c, io.c, upd.c, med.c, compiled from the reference tree by
// oracle/Makefile, target ref-host) and dumps what it computes, so that
// tests/golden/ can pin the oracle against the reference itself:
//   seeds, generator states, geometry tables, packed spins and couplings,
//   scalar energies, the Philox counters of the first half-sweeps
//   (fill_bits.h), and Parallel_Tempering decisions on synthetic energies.
// Geometry comes from the reference's compile-time macros (L, Lz, NBETAS,
// PBC/OBC/WEAK/STRONG); the header declares its globals `extern`, and this
// file provides their definitions plus a driver.
#include "header.h"
#include "fill_bits.h"
#include <stdint.h>

int list_samples[MAXNSAMPLES];
int x_p[Lx], x_m[Lx], y_p[Ly], y_m[Ly], z_p[Lz], z_m[Lz];
Vicini viciniB[HALF_MSC_V], viciniN[HALF_MSC_V];
unsigned int bianchi_index[HALF_MSC_V], neri_index[HALF_MSC_V];
unsigned char bianchi_rotate[HALF_MSC_V], neri_rotate[HALF_MSC_V];
int side[DIM], off[DIM + 1];
int numThreadsPerBlock, numBlocks;
s_data data;
int write_seeds;
double betas[NBETAS];
int countJ0[MAXNSAMPLES];
s_lut_heat_bath h_LUT[NBETAS];
s_keys seed_keys;
s_time s_time_and_entropy;
randint seeds_J[MAXNSAMPLES], seeds_u[MAXNSAMPLES], seeds_MC[NR];
s_aleatorio_HQ_64bits random_u, random_J, random_c;
s_aleatorio_HQ_64bits random_PRC[NR], random_PT[MAXNSAMPLES][NR];
s_xoshiro256pp random_xoshiro256pp[NR];
uint64_t cuda_rng_offset;
char ***uu[MAXNSAMPLES], *Jx[MAXNSAMPLES], *Jy[MAXNSAMPLES], *Jz[MAXNSAMPLES];
char *Jmx[MAXNSAMPLES], *Jmy[MAXNSAMPLES], *Jmz[MAXNSAMPLES];
MYWORD *h_MSC_u_even[MAXNSAMPLES], *h_MSC_u_odd[MAXNSAMPLES];
int *h_Ener;
double aceptancePT[MAXNSAMPLES][NR][NBETAS - 1], attemptsPT[MAXNSAMPLES][NR][NBETAS - 1],
    aceptancePTraw[MAXNSAMPLES][NR][NBETAS - 1];
uint8_t which_clon_this_beta[MAXNSAMPLES][NR][NBETAS];
uint8_t which_beta_this_clon[MAXNSAMPLES][NR][NBETAS];
double average_Energy[MAXNSAMPLES][NRNBETAS];
int frecTRW, maxit_TRW;
unsigned char history_betas[MAXNSAMPLES][NR][MAXIT_TRW][NBETAS];
int sum[MAX];

static FILE *out;
static void put(const char *name, const void *p, size_t bytes) {
  uint32_t n = (uint32_t)strlen(name);
  uint64_t b = bytes;
  fwrite(&n, 4, 1, out);
  fwrite(name, 1, n, out);
  fwrite(&b, 8, 1, out);
  fwrite(p, 1, bytes, out);
}

// usage: harness outdir nbits seedJ seedu seedMC seedC betasfile outfile
int main(int argc, char **argv) {
  if (argc != 9) { fprintf(stderr, "usage: %s dir nbits sJ su sMC sC betas out\n", argv[0]); return 1; }
  int nbits = atoi(argv[2]);
  char input[MAXSTR];
  snprintf(input, MAXSTR, "%s/input.in", argv[1]);
  FILE *f = fopen(input, "w");
  fprintf(f, "%s/\n1\n0\n1\n1\n1\n1\n%d\n1\n%d\n%s\n%s\n%s\n%s\n", argv[1], NBETAS, (Lz << 16) | L,
          argv[3], argv[4], argv[5], argv[6]);
  fclose(f);
  read_input(input);
  read_betas(argv[7]);
  read_list_samples("", nbits);
  create_sample_path(0, nbits);
  check_and_prepare_simulation_backup(0, nbits);
  for (int ib = 0; ib < nbits; ib++) {
    Jx[ib] = (char *)malloc(V); Jy[ib] = (char *)malloc(V); Jz[ib] = (char *)malloc(V);
    Jmx[ib] = (char *)malloc(V); Jmy[ib] = (char *)malloc(V); Jmz[ib] = (char *)malloc(V);
    h_MSC_u_even[ib] = (MYWORD *)malloc(sizeof(MYWORD) * HALF_MSC_VNRNBETAS);
    h_MSC_u_odd[ib] = (MYWORD *)malloc(sizeof(MYWORD) * HALF_MSC_VNRNBETAS);
    uu[ib] = (char ***)malloc(sizeof(char **) * NR);
    for (int r = 0; r < NR; r++) {
      uu[ib][r] = (char **)malloc(sizeof(char *) * NBETAS);
      for (int c = 0; c < NBETAS; c++) uu[ib][r][c] = (char *)malloc(V);
    }
  }
  Init(nbits);

  out = fopen(argv[8], "wb");
  int geom[6] = {L, Lz, NBETAS, NR, nbits, 0};
  put("geom", geom, sizeof(geom));
  put("seeds_J", seeds_J, sizeof(randint) * nbits);
  put("seeds_u", seeds_u, sizeof(randint) * nbits);
  put("seeds_MC", seeds_MC, sizeof(randint) * NR);
  put("keys", seed_keys.my_key, sizeof(uint32_t) * NR);
  put("prc", random_PRC, sizeof(random_PRC));
  put("xo", random_xoshiro256pp, sizeof(random_xoshiro256pp));
  put("rc", &random_c, sizeof(random_c));
  for (int ib = 0; ib < nbits; ib++) {
    char nm[64];
    snprintf(nm, 64, "pt%d", ib); put(nm, random_PT[ib], sizeof(random_PT[ib]));
    snprintf(nm, 64, "even%d", ib); put(nm, h_MSC_u_even[ib], sizeof(MYWORD) * HALF_MSC_VNRNBETAS);
    snprintf(nm, 64, "odd%d", ib); put(nm, h_MSC_u_odd[ib], sizeof(MYWORD) * HALF_MSC_VNRNBETAS);
    static char J6[6 * V];
    memcpy(J6, Jx[ib], V); memcpy(J6 + V, Jy[ib], V); memcpy(J6 + 2 * V, Jz[ib], V);
    memcpy(J6 + 3 * V, Jmx[ib], V); memcpy(J6 + 4 * V, Jmy[ib], V); memcpy(J6 + 5 * V, Jmz[ib], V);
    snprintf(nm, 64, "J6_%d", ib); put(nm, J6, 6 * V);
    static MYWORD Jw[2 * DEGREE * HALF_MSC_V];
    for (int p = 0; p < 2; p++)
      for (int d = 0; d < DEGREE; d++)
        for (int k = 0; k < HALF_MSC_V; k++)
          Jw[(p * DEGREE + d) * HALF_MSC_V + k] = (p ? viciniN : viciniB)[k].J[ib][d];
    snprintf(nm, 64, "Jw%d", ib); put(nm, Jw, sizeof(Jw));
    static int32_t escal[NR * NBETAS];
    for (int r = 0; r < NR; r++)
      for (int c = 0; c < NBETAS; c++) escal[r * NBETAS + c] = calculate_scalar_energy(ib, r, c);
    snprintf(nm, 64, "escalar%d", ib); put(nm, escal, sizeof(escal));
  }
  static int32_t neig[2 * DEGREE * HALF_MSC_V];
  for (int p = 0; p < 2; p++)
    for (int d = 0; d < DEGREE; d++)
      for (int k = 0; k < HALF_MSC_V; k++) neig[(p * DEGREE + d) * HALF_MSC_V + k] = (p ? viciniN : viciniB)[k].neig[d];
  put("neig", neig, sizeof(neig));
  put("rot_even", bianchi_rotate, HALF_MSC_V);
  put("rot_odd", neri_rotate, HALF_MSC_V);
  put("bianchi", bianchi_index, sizeof(bianchi_index));
  put("neri", neri_index, sizeof(neri_index));

  // Philox counters of 6 consecutive half-sweeps starting at iter0 (fill_bits.h:47-68)
  {
    const int NH = 6;
    static uint32_t ctr[NH][NR][4];
    int ir;
    uint64_t entropy, temporal, parity;
    uint32_t mi_jobID = 37;
    int iter = 1000;
    for (int h = 0; h < NH; h++) {
      parity = (uint64_t)(iter & 1);
      _fill_bits;
      for (int r = 0; r < NR; r++) {
        ctr[h][r][0] = s_time_and_entropy.vec[r].x; ctr[h][r][1] = s_time_and_entropy.vec[r].y;
        ctr[h][r][2] = s_time_and_entropy.vec[r].z; ctr[h][r][3] = s_time_and_entropy.vec[r].w;
      }
      iter++;
    }
    put("ctr_iter1000_job37", ctr, sizeof(ctr));
  }

  // Parallel_Tempering on synthetic energies, 5 rounds per (sample, replica)
  {
    static int32_t ener[NBETAS];
    static uint8_t perm_after[MAXNSAMPLES][NR][5][NBETAS];
    static int32_t energies_used[MAXNSAMPLES][NR][5][NBETAS];
    uint64_t lcg = 12345;
    for (int ib = 0; ib < nbits; ib++)
      for (int r = 0; r < NR; r++)
        for (int round = 0; round < 5; round++) {
          for (int c = 0; c < NBETAS; c++) {
            lcg = lcg * 6364136223846793005ULL + 1442695040888963407ULL;
            ener[c] = -(int32_t)(V) + (int32_t)((lcg >> 33) % (uint64_t)(V / 4)) * 2;
          }
          memcpy(energies_used[ib][r][round], ener, sizeof(ener));
          Parallel_Tempering(&random_PT[ib][r], which_clon_this_beta[ib][r], which_beta_this_clon[ib][r], ener,
                             aceptancePT[ib][r], attemptsPT[ib][r], aceptancePTraw[ib][r]);
          memcpy(perm_after[ib][r][round], which_clon_this_beta[ib][r], NBETAS);
        }
    put("pt_energies", energies_used, sizeof(int32_t) * nbits * NR * 5 * NBETAS);
    put("pt_perm", perm_after, (size_t)nbits * NR * 5 * NBETAS);
    put("pt_acc", aceptancePT, sizeof(double) * nbits * NR * (NBETAS - 1));
    put("pt_accraw", aceptancePTraw, sizeof(double) * nbits * NR * (NBETAS - 1));
    put("pt_state_after", random_PT, sizeof(s_aleatorio_HQ_64bits) * nbits * NR);
  }
  fclose(out);
  return 0;
}
