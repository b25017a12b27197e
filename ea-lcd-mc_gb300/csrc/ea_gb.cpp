// ea_gb.cpp -- command-line driver with the reference's interface
// (PROGRAM/src/main.cu:10-283 and PROGRAM/src/io.c):
//
//   ea_gb isample nbits beta.dat input.in LUT device [max_time [list_samples]]
//
// It reads the same input, betas, LUT and sample-list files and writes the
// same output tree and file formats (couplings.bin, seeds.in, master_seeds.in,
// conf.%06d + conf, evol.txt, aceptancePT.txt, history_b.dat, run.log,
// running, error), with the same restart flags, lock file, signal handling,
// changenbin.in and time budget.  The simulation itself runs through the C ABI
// of libeagb.so on the GPU.
//
// The reference fixes L, Lz, NBETAS, the boundary condition and the cluster
// move at compile time and names its executables accordingly
// (PROGRAM/Makefile:140, e.g. EA_CUBE_L16_Lz48_NB40_NBPRE12_OBC).  When this
// program is invoked under such a name (a symbolic link), it takes the boundary
// condition and NO_CLUSTER from the name and checks L, Lz and NBETAS against
// the input file as the reference does; otherwise EAGB_BC (PBC, OBC, WEAK,
// STRONG; default OBC) and EAGB_NO_CLUSTER=1 select them.
//
// Output location: the reference builds the sample directory with
// sprintf(dir, "%sI%03d/", dir, sample) (io.c:573); with glibc the source
// string is lost and the tree lands in ./I%03d/ under the working directory.
// This driver writes it there too, so existing scripts find the files.
#include <cmath>
#include <csignal>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

#include "eagb.h"

namespace {

constexpr int kNR = 8;
constexpr int kMaxSamples = 32;
constexpr int kMaxNbin = 4096;
constexpr int kMaxStr = 1024;

struct Data {
  int32_t nbin = 0, itcut = 0, itmax = 0, houfr = 0, mesfr = 0, ptfr = 0, nbetas = 0, flag = 0, l = 0;
  uint64_t seed_J = 0, seed_u = 0, seed_MC = 0, seed_C = 0;
};

Data data;
std::string dir;
std::vector<std::string> dirsample;
std::vector<std::vector<std::string>> dir_rep;
char host[100];
int pid;

[[noreturn]] void print_and_exit(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  exit(1);
}

void print_data(FILE *f, const Data &d) {
  fprintf(f, "nbin        %16d\n", d.nbin);
  fprintf(f, "itcut       %16d\n", d.itcut);
  fprintf(f, "itmax       %16d\n", d.itmax);
  fprintf(f, "houfr       %16d\n", d.houfr);
  fprintf(f, "mesfr       %16d\n", d.mesfr);
  fprintf(f, "ptfr        %16d\n", d.ptfr);
  fprintf(f, "flag        %16d\n", d.flag);
  fprintf(f, "L           %16d\n", d.l & 0xffff);
  fprintf(f, "M           %16d\n", d.l >> 16);
  fprintf(f, "nbetas      %16d\n", d.nbetas);
  fprintf(f, "Master seeds:\n");
  fprintf(f, "seed_J      %016llx\n", (unsigned long long)d.seed_J);
  fprintf(f, "seed_u      %016llx\n", (unsigned long long)d.seed_u);
  fprintf(f, "seed_MC     %016llx\n", (unsigned long long)d.seed_MC);
  fprintf(f, "seed_Cl     %016llx\n", (unsigned long long)d.seed_C);
}

void delete_running() { remove((dir + "/running").c_str()); }

// create_error (io.c:920-938): message and data into <dir>/error.
void create_error(const char *fmt, ...) {
  FILE *f = fopen((dir + "/error").c_str(), "w");
  va_list ap;
  va_start(ap, fmt);
  if (f) vfprintf(f, fmt, ap);
  va_end(ap);
  if (f) { print_data(f, data); fclose(f); }
  print_data(stderr, data);
  delete_running();
}

// The reference's handler writes <dir>/error and exits 1 (io.c:894-918).  The
// signal can interrupt a CUDA runtime call that holds the runtime's locks, so
// the process ends with _exit after flushing its streams: exit() would run the
// runtime's teardown from inside the handler, which can wait on those locks
// for ever.  The driver releases the device when the process ends.
void stop_run(int sig) {
  if (sig == SIGTERM) create_error("Received SIGTERM\n");
  if (sig == SIGINT) create_error("Received SIGINT\n");
  if (sig == SIGUSR1) create_error("Received SIGUSR1\n");
  fprintf(stderr, "Aborting programma (SIGNAL=%d)\n", sig);
  fflush(stdout);
  fflush(stderr);
  _exit(1);
}

void ignore_sigterm() { signal(SIGTERM, SIG_IGN); signal(SIGINT, SIG_IGN); signal(SIGUSR1, SIG_IGN); }
void handle_sigterm() { signal(SIGTERM, stop_run); signal(SIGINT, stop_run); signal(SIGUSR1, stop_run); }

void writelog(FILE *f, time_t t) { fprintf(f, "%s %5d %10ld %s", host, pid, (long)t, ctime(&t)); }

// create_running / renew_running (io.c:940-1004): a lock made atomic by link().
void create_running() {
  gethostname(host, 99);
  pid = getpid();
  char name[kMaxStr];
  snprintf(name, sizeof(name), "%srunning.%s.%d", dir.c_str(), host, pid);
  const std::string link_name = dir + "running";
  FILE *f = fopen(name, "w");
  if (!f) print_and_exit("Unable to open %s\n", name);
  writelog(f, time(nullptr));
  fclose(f);
  if (link(name, link_name.c_str()) == -1) {
    remove(name);
    print_and_exit("%s exists\n", link_name.c_str());
  }
  remove(name);
  FILE *lg = fopen((dir + "run.log").c_str(), "a");
  if (!lg) print_and_exit("Unable to open %srun.log\n", dir.c_str());
  writelog(lg, time(nullptr));
  fclose(lg);
}

void renew_running() {
  const std::string name = dir + "/running";
  FILE *f = fopen(name.c_str(), "r+");
  if (!f) {
    create_error("File %s doesn't exist\n", name.c_str());
    print_and_exit("File %s doesn't exist\n", name.c_str());
  }
  char h[100] = {0};
  int p = 0;
  if (fscanf(f, "%99s %d", h, &p) != 2) h[0] = 0;
  if (strcmp(host, h)) {
    create_error("Host has changed from %s to %s\n", host, h);
    print_and_exit("Host has changed from %s to %s\n", host, h);
  }
  if (p != pid) {
    create_error("PID has changed from %d to %d\n", pid, p);
    print_and_exit("PID has changed from %d to %d\n", pid, p);
  }
  rewind(f);
  writelog(f, time(nullptr));
  fclose(f);
}

// stop (io.c:870-891): <dir>changenbin.in overrides nbin and is removed.
void stop(int *nbin) {
  const std::string name = dir + "changenbin.in";
  FILE *f = fopen(name.c_str(), "r");
  if (!f) return;
  if (fscanf(f, "%d", nbin) == EOF) {
    *nbin = -1;
    printf(" File '%s' exists\n", name.c_str());
  }
  if (*nbin > kMaxNbin) {
    create_error(" nbin must be smaller than %d\n", kMaxNbin);
    print_and_exit(" nbin must be smaller than %d\n", kMaxNbin);
  }
  fclose(f);
  printf("nbin changed to %d\n", *nbin);
  fflush(stdout);
  remove(name.c_str());
}

// measure_time (timing.c:3-41): wall time and ps per spin update of each bin.
void measure_time(double totalspins_per_bin) {
  static timespec wall0 = {0, 0}, cpu0;
  timespec wall1, cpu1;
  clock_gettime(CLOCK_MONOTONIC, &wall1);
  clock_gettime(CLOCK_PROCESS_CPUTIME_ID, &cpu1);
  if (wall0.tv_sec > 0) {
    const double el = (wall1.tv_sec - wall0.tv_sec) * 1e9 + (wall1.tv_nsec - wall0.tv_nsec);
    const double cp = (cpu1.tv_sec - cpu0.tv_sec) * 1e9 + (cpu1.tv_nsec - cpu0.tv_nsec);
    printf("%4.0fs (%.3f ps/s, %.0f%%): ", el * 1e-9, el / totalspins_per_bin * 1e3, cp / el * 100);
  } else {
    printf("Starting simulation\n");
  }
  wall0 = wall1;
  cpu0 = cpu1;
}

// check_time (timing.c:43-74): stop when mean + 3 sigma of a bin no longer fits.
int check_time(unsigned long long max_time) {
  static timespec t0 = {0, 0};
  static unsigned total = 0, el2 = 0, n = 0;
  timespec t1;
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (t0.tv_sec > 0 && max_time != 0) {
    const unsigned el = (unsigned)(t1.tv_sec - t0.tv_sec);
    total += el;
    el2 += el * el;
    n++;
    const double mean = (double)total / n;
    double sd = (double)el2 / n;
    sd = n > 1 ? std::sqrt(n * (sd - mean * mean) / ((double)n - 1)) : 0.0;
    const unsigned next = (unsigned)(mean + 3 * sd + 1);
    if (((double)max_time) - total - next <= 0) return 1;
  }
  t0 = t1;
  return 0;
}

uint64_t urandom64() {
  uint64_t v = 0;
  FILE *f = fopen("/dev/urandom", "r");
  if (f) { if (fread(&v, sizeof(v), 1, f) != 1) v = 0; fclose(f); }
  return v;
}

uint64_t check_seed(uint64_t s) { return s ? s : urandom64(); }  // comprueba_semilla

void ck(int rc, const char *what) {
  if (rc != EA_OK) {
    fprintf(stderr, "%s failed: %s\n", what, ea_last_error());
    exit(EXIT_FAILURE);
  }
}

// Boundary condition, cluster switch and compile-time sizes from a reference
// executable name: EA_CUBE_L<L>_Lz<Lz>_NB<NB>_NBPRE<n>_<BC>[_NO_CLUSTER].
struct Build {
  int bc = EA_OBC, cluster = 1, L = 0, Lz = 0, NB = 0;
};

Build build_from_name(const char *argv0) {
  Build b;
  const char *base = strrchr(argv0, '/');
  base = base ? base + 1 : argv0;
  int L, Lz, NB, npre, n = 0;
  if (sscanf(base, "EA_CUBE_L%d_Lz%d_NB%d_NBPRE%d%n", &L, &Lz, &NB, &npre, &n) == 4) {
    b.L = L; b.Lz = Lz; b.NB = NB;
    const std::string rest = base + n;
    if (rest.find("_PBC") == 0) b.bc = EA_PBC;
    else if (rest.find("_OBC_WEAK") == 0) b.bc = EA_OBC_WEAK;
    else if (rest.find("_OBC_STRONG") == 0) b.bc = EA_OBC_STRONG;
    else b.bc = EA_OBC;
    if (rest.find("_NO_CLUSTER") != std::string::npos) b.cluster = 0;
    return b;
  }
  if (const char *e = getenv("EAGB_BC")) {
    if (!strcmp(e, "PBC")) b.bc = EA_PBC;
    else if (!strcmp(e, "WEAK")) b.bc = EA_OBC_WEAK;
    else if (!strcmp(e, "STRONG")) b.bc = EA_OBC_STRONG;
    else b.bc = EA_OBC;
  }
  if (const char *e = getenv("EAGB_NO_CLUSTER")) b.cluster = atoi(e) ? 0 : 1;
  return b;
}

void print_help(const char *prog) {
  printf("Usage: %s isample ibit beta.dat input.in LUT device [max_time [list_samples]]\n", prog);
  printf("\nArguments:\n");
  printf("  isample              Sample index (int)\n");
  printf("  nbits                Number of subsample (int)\n");
  printf("  beta.dat             Path to beta.dat file (string)\n");
  printf("  input.in             Path to input.in file (string)\n");
  printf("  LUT                  Path to LUT file (string)\n");
  printf("  device               Device number (int)\n");
  printf("  max_time (opt.)      Maximum time allowed (unsigned long long)\n");
  printf("                       A 0 value disable this option.\n");
  printf("  list_samples (opt.)  oPath to the list_of_samples file (string)\n");
  printf("\nUse -h to display this help message.\n");
  exit(EXIT_SUCCESS);
}

void write_file(const std::string &path, const void *p, size_t n) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) print_and_exit("Problems opening %s\n", path.c_str());
  fwrite(p, 1, n, f);
  fclose(f);
}

}  // namespace

int main(int argc, char **argv) {
  if (argc > 1 && (!strcmp(argv[1], "-h") || !strcmp(argv[1], "--help"))) print_help(argv[0]);
  int sample = 0, nbits = 0, device = 0;
  unsigned long long max_time = 0;
  std::string name_list, name_lut, name_input, name_betas;
  check_time(max_time);
  switch (argc) {
    case 9: name_list = argv[8]; [[fallthrough]];
    case 8: sscanf(argv[7], "%llu", &max_time); [[fallthrough]];
    case 7:
      sscanf(argv[6], "%d", &device);
      name_lut = argv[5];
      name_input = argv[4];
      name_betas = argv[3];
      sscanf(argv[2], "%d", &nbits);
      sscanf(argv[1], "%d", &sample);
      break;
    default:
      print_and_exit("Usage: %s isample nbits beta.dat input.in LUT device [max_time [list_samples]]\n", argv[0]);
  }
  if (nbits < 0 || nbits >= kMaxSamples) print_and_exit("Error: nbits out of range, 0 <= bit < %d\n", kMaxSamples);
  if (sample < 0) print_and_exit("Error: sample out of range, 0 <= sample\n");
  const uint32_t jobid = (uint32_t)sample;
  if (jobid > (1u << 14) - 1) print_and_exit("Our Counter-based PRNG  cannot accomodate more than %d samples\n", 1 << 14);
  const Build bld = build_from_name(argv[0]);
  {
    int32_t ndev = 0;
    ck(ea_device_count(&ndev), "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) print_and_exit("device=%d count_devices=%d\n", device, ndev);
  }

  // read_input (io.c:399-436)
  {
    FILE *f = fopen(name_input.c_str(), "r");
    if (!f) print_and_exit("Error: No file %s\n", name_input.c_str());
    char line[kMaxStr + 1], buf[kMaxStr];
    if (!fgets(line, kMaxStr, f) || sscanf(line, "%1023s", buf) != 1) print_and_exit("Bad data input\n");
    dir = buf;
    int32_t *fields[9] = {&data.nbin, &data.itcut, &data.itmax, &data.houfr, &data.mesfr, &data.ptfr, &data.nbetas, &data.flag, &data.l};
    for (auto *p : fields) {
      unsigned v = 0;
      if (!fgets(line, kMaxStr, f) || sscanf(line, "%u", &v) != 1) print_and_exit("Bad data input\n");
      *p = (int32_t)v;
    }
    uint64_t *seeds[4] = {&data.seed_J, &data.seed_u, &data.seed_MC, &data.seed_C};
    for (auto *p : seeds) {
      unsigned long long v = 0;
      if (!fgets(line, kMaxStr, f) || sscanf(line, "%llu", &v) != 1) print_and_exit("Bad data input\n");
      *p = v;
    }
    fclose(f);
  }
  auto check_data = [&](const Data &d) {
    if (d.nbin < 0 || d.itcut < 0 || d.itmax < 0 || d.houfr < 0 || d.mesfr < 0 || d.ptfr < 0) print_and_exit("Bad data input\n");
    if (bld.NB && d.nbetas != bld.NB) print_and_exit("d.nbetas = %d != NBETAS = %d\n", d.nbetas, bld.NB);
    if (bld.L && (d.l & 0xffff) != bld.L) print_and_exit("l=%d != L=%d\n", d.l & 0xffff, bld.L);
    if (bld.Lz && (d.l >> 16) != bld.Lz) print_and_exit("lz=%d != M=%d\n", d.l >> 16, bld.Lz);
    if (d.ptfr >= 1000) print_and_exit("The number(%d) of Metropolis per PT is too large\n", d.ptfr);
  };
  check_data(data);
  printf("Path: %s\n", dir.c_str());
  print_data(stdout, data);
  fflush(stdout);
  const int L = data.l & 0xffff, Lz = data.l >> 16, NB = data.nbetas, NR = kNR;
  ea_geom geo{L, Lz, NB, NR, nbits > 0 ? nbits : 1, bld.bc};
  {
    ea_geom probe = geo;
    std::vector<uint64_t> e(1), o(1);
    if (L % 8 || Lz % 8 || L < 8 || Lz < 8) print_and_exit("L=%d and Lz=%d must be multiples of 8\n", L, Lz);
    if (NB < 2 || NB > 255) print_and_exit("d.nbetas = %d out of range\n", NB);
    (void)probe;
  }
  int frec = 1, maxit = data.itmax;
  for (frec = 1; frec <= data.itmax; frec++)
    if (data.itmax % frec == 0 && (maxit = data.itmax / frec) <= 512) break;

  // read_betas (io.c:476-501)
  std::vector<double> betas(NB);
  {
    FILE *f = fopen(name_betas.c_str(), "rt");
    if (!f) print_and_exit("File  %s doesn't exist.\n", name_betas.c_str());
    for (int i = 0; i < NB; i++)
      if (fscanf(f, "%lf ", &betas[i]) == EOF) print_and_exit("File %s only has %d lines (it needs %d)\n", name_betas.c_str(), i, NB);
    double dummy;
    if (fscanf(f, "%lf", &dummy) != EOF) fprintf(stderr, "More lines in file %s\n", name_betas.c_str());
    for (int i = 0; i + 1 < NB; i++)
      if (betas[i] < betas[i + 1]) print_and_exit("Error in file %s: betas don't sort from largest to smallest!\n", name_betas.c_str());
    fclose(f);
  }
  // read_lut (io.c:504-534): betas, then per beta 128 uint4 thresholds and the pre-search table
  std::vector<uint64_t> cum((size_t)NB * 256);
  {
    FILE *f = fopen(name_lut.c_str(), "rb");
    if (!f) print_and_exit("Problems opening %s\n", name_lut.c_str());
    std::vector<double> bl(NB, 0.0);
    if (fread(bl.data(), sizeof(double) * NB, 1, f) != 1) {
      printf("betas_read[0]=%.14g\n", bl[0]);
      printf("betas_read[1]=%.14g\n", NB > 1 ? bl[1] : 0.0);
      print_and_exit("Problems reading betas\n");
    }
    for (int i = 0; i < NB; i++)
      if (std::fabs(betas[i] - bl[i]) > 1e-14)
        print_and_exit("betas[%d]=%.14g from %s, betas[%d]=%.14g from %s (difference=%.14g)\n", i, betas[i],
                       name_betas.c_str(), i, bl[i], name_lut.c_str(), betas[i] - bl[i]);
    std::vector<uint32_t> rec((128 + 512) * 4);
    for (int b = 0; b < NB; b++) {
      if (fread(rec.data(), rec.size() * 4, 1, f) != 1) print_and_exit("Problems reading lut_heat_bath\n");
      for (int n = 0; n < 256; n++) cum[(size_t)b * 256 + n] = ((uint64_t)rec[2 * n] << 32) | rec[2 * n + 1];
    }
    fclose(f);
  }
  // read_list_samples (io.c:536-567)
  std::vector<int32_t> list(nbits);
  if (name_list.empty()) {
    for (int i = 0; i < nbits; i++) list[i] = i;
  } else {
    FILE *f = fopen(name_list.c_str(), "rt");
    if (!f) print_and_exit("File  %s doesn't exist.\n", name_list.c_str());
    for (int i = 0; i < nbits; i++)
      if (fscanf(f, "%d ", &list[i]) == EOF) print_and_exit("File %s only has %d lines (it needs %d)\n", name_list.c_str(), i, nbits);
    int dummy;
    if (fscanf(f, "%d", &dummy) != EOF) fprintf(stderr, "More lines in file %s\n", name_list.c_str());
    fclose(f);
  }
  for (int i = 0; i + 1 < nbits; i++)
    if (list[i] >= list[i + 1]) {
      create_error("List of samples %s is not sorted.\n", name_list.c_str());
      print_and_exit("List of samples must be sorted!\n");
    }
  for (int i = 0; i < nbits; i++)
    if (list[i] < 0 || list[i] >= kMaxSamples) print_and_exit("Sample %d of the list is outside [0, %d)\n", list[i], kMaxSamples);

  // create_sample_path (io.c:569-589), with the working-directory placement described above
  {
    char buf[kMaxStr];
    snprintf(buf, sizeof(buf), "I%03d/", sample);
    dir = buf;
    mkdir(dir.c_str(), 0775);
    dirsample.resize(nbits);
    dir_rep.assign(nbits, std::vector<std::string>(NR));
    for (int i = 0; i < nbits; i++) {
      snprintf(buf, sizeof(buf), "%sBIT%03d/", dir.c_str(), list[i]);
      dirsample[i] = buf;
      mkdir(buf, 0775);
      for (int r = 0; r < NR; r++) {
        snprintf(buf, sizeof(buf), "%sR%02d/", dirsample[i].c_str(), r);
        dir_rep[i][r] = buf;
        mkdir(buf, 0775);
      }
    }
    printf("Dirsample = %s\n", dir.c_str());
    fflush(stdout);
  }

  // check_and_prepare_simulation_backup + get_seeds (io.c:598-809)
  int there_is_conf = 0, check_itcut = 0, itcut_seen = 0;
  for (int i = 0; i < nbits; i++) {
    there_is_conf = 0;
    for (int r = 0; r < NR; r++) {
      FILE *f = fopen((dir_rep[i][r] + "/conf").c_str(), "r");
      if (!f) continue;
      int32_t hdr[9] = {0};
      if (fread(hdr, 4, 9, f) != 9) hdr[1] = -1;
      if (check_itcut > 0 && hdr[1] != itcut_seen) {
        create_error("Different number of iterations in samples from %s\n", dir.c_str());
        print_and_exit("Problems with conf files\n");
      }
      itcut_seen = hdr[1];
      there_is_conf++;
      check_itcut++;
      fclose(f);
    }
    if (there_is_conf > 0 && there_is_conf != NR) {
      create_error("There are less conf files than it must be in %s (%d/%d)\n", dirsample[i].c_str(), there_is_conf, NR);
      print_and_exit("Problems with conf files\n");
    }
  }
  if (data.flag == 2) data.flag = there_is_conf ? 0 : 1;
  if (data.flag == 1) {
    if (there_is_conf) {
      create_error("There are some confs in %s.\nIf you want to make a new run, please delete the configuration manually\n", dir.c_str());
      print_and_exit("There are confs\n");
    }
  } else if (data.flag == 0) {
    if (there_is_conf == 0) {
      create_error("There is not %s/conf, it is impossible to do a backup\n", nbits ? dir_rep[nbits - 1][NR - 1].c_str() : dir.c_str());
      print_and_exit("Impossible to do a backup\n");
    }
  } else {
    print_and_exit("data.flag is not recognize\n");
  }
  std::vector<uint64_t> seeds_J(nbits), seeds_u(nbits), seeds_MC(NR);
  std::vector<int32_t> countJ0(nbits, 0);
  int write_seeds = 0;
  {
    int no_master = 0, no_seeds = 0;
    const std::string mname = dir + "/master_seeds.in";
    FILE *f = fopen(mname.c_str(), "r");
    if (!f) {
      if (data.flag == 1) no_master = 1;
      else {
        sleep(1);
        if (!(f = fopen(mname.c_str(), "r"))) {
          create_error("There is not file %s, and it must exist\n", mname.c_str());
          print_and_exit("Problems reading seeds\n");
        }
      }
    }
    if (!no_master) {
      unsigned long long sJ, su, sMC, sC;
      if (fscanf(f, "%llu %llu %llu %llu", &sJ, &su, &sMC, &sC) == EOF) print_and_exit("Nothing in file %s\n", mname.c_str());
      fclose(f);
      auto take = [&](uint64_t &dst, unsigned long long v, const char *what) {
        if (dst > 0 && dst != v) {
          create_error("Master seed%s in input file and %s differ\n", what, mname.c_str());
          print_and_exit("Problems reading master seedJ\n");
        }
        dst = v;
      };
      take(data.seed_J, sJ, "J");
      take(data.seed_u, su, "u");
      take(data.seed_MC, sMC, "MC");
      take(data.seed_C, sC, "Cluster");
    }
    const bool u_elim = data.flag == 0 && data.seed_u == 0, mc_elim = data.flag == 0 && data.seed_MC == 0;
    data.seed_J = check_seed(data.seed_J);
    data.seed_u = check_seed(data.seed_u);
    data.seed_MC = check_seed(data.seed_MC);
    ck(ea_host_seeds(data.seed_J, data.seed_u, data.seed_MC, data.seed_C, list.data(), nbits > 0 ? nbits : 1, NR,
                     seeds_J.data(), seeds_u.data(), seeds_MC.data()),
       "seed derivation");
    if (u_elim) data.seed_u = 0;
    if (mc_elim) data.seed_MC = 0;
    for (int i = 0; i < nbits; i++) {
      const std::string sname = dirsample[i] + "/seeds.in";
      FILE *g = fopen(sname.c_str(), "r");
      if (!g) {
        if (data.flag == 1) { no_seeds++; continue; }
        sleep(1);
        if (!(g = fopen(sname.c_str(), "r"))) {
          create_error("There is not file %s, and it must exist\n", sname.c_str());
          print_and_exit("Problems reading seeds\n");
        }
      }
      unsigned long long sJ = 0, su = 0, sMC[kNR] = {0}, sC = 0;
      int n = fscanf(g, "%llu %llu", &sJ, &su);
      for (int r = 0; r < NR; r++) n += fscanf(g, " %llu", &sMC[r]);
      n += fscanf(g, " %llu", &sC);
      n += fscanf(g, " %d", &countJ0[i]);
      fclose(g);
      if (n != NR + 4) {
        create_error("File %s must have %d fields\n", sname.c_str(), NR + 4);
        print_and_exit("Problems reading seeds from %s\n", sname.c_str());
      }
      if (seeds_J[i] != sJ) {
        create_error("Seed J generated and %s differ (bit=%d)\n", sname.c_str(), list[i]);
        print_and_exit("Problems reading seeds\n");
      }
      if (seeds_u[i] != su && su != 0 && !u_elim) {
        create_error("Seed u generated and %s differ (bit=%d)\n", sname.c_str(), list[i]);
        print_and_exit("Problems reading seeds\n");
      }
      seeds_u[i] = su;
      for (int r = 0; r < NR; r++) {
        if (seeds_MC[r] != sMC[r] && sMC[r] != 0 && !mc_elim) {
          create_error("Seed MC generated input and %s differ\n", sname.c_str());
          print_and_exit("Problems reading seeds\n");
        }
        seeds_MC[r] = sMC[r];
      }
    }
    if (no_seeds == nbits || no_master) write_seeds = 1;
    else if (no_seeds > 0) print_and_exit("Some samples have file seeds.in, others not have\n");
  }
  printf("Betas and LUT have been read correctly.\n");
  printf("Initializating J's and Spins ...\n");
  fflush(stdout);
  handle_sigterm();
  create_running();

  // Init (ini.c:8-30): generators, spins, couplings, permutations
  for (auto &s : seeds_MC) s = check_seed(s);
  for (int i = 0; i < nbits; i++) { seeds_J[i] = check_seed(seeds_J[i]); seeds_u[i] = check_seed(seeds_u[i]); }
  data.seed_C = check_seed(data.seed_C);
  ea_generators gen;
  std::vector<ea_hq> pt((size_t)(nbits > 0 ? nbits : 1) * NR);
  ck(ea_host_generators(seeds_MC.data(), list.data(), nbits > 0 ? nbits : 1, NR, data.seed_C, &gen, pt.data()), "generators");
  const size_t half = (size_t)(L / 4) * (L / 4) * (Lz / 4) / 2, V = (size_t)L * L * Lz, nw = (size_t)NB * half * NR;
  std::vector<std::vector<uint64_t>> ev(nbits, std::vector<uint64_t>(nw)), od(nbits, std::vector<uint64_t>(nw));
  std::vector<std::vector<uint64_t>> Jw(nbits, std::vector<uint64_t>(12 * half));
  std::vector<std::vector<uint8_t>> J6(nbits, std::vector<uint8_t>(6 * V));
  for (int i = 0; i < nbits; i++) ck(ea_host_init_spins(&geo, seeds_u[i], ev[i].data(), od[i].data()), "spins");
  printf("Packing spins well done.\n");
  printf("J random\n");
  for (int i = 0; i < nbits; i++) {
    int32_t cnt = 0;
    ck(ea_host_init_couplings(&geo, seeds_J[i], J6[i].data(), Jw[i].data(), &cnt), "couplings");
    if (data.flag == 0 && cnt != countJ0[i]) {
      create_error("countJ and countJ0 differ (%d != %d --- ibit=%d)\n", cnt, countJ0[i], list[i]);
      print_and_exit("Problems generating J's\n");
    }
    if (countJ0[i] != 0 && countJ0[i] != cnt) {
      create_error("CountJ and countJ0 differ\n");
      print_and_exit("Problems generating J's\n");
    }
    countJ0[i] = cnt;
    write_file(dirsample[i] + "/couplings.bin", J6[i].data(), J6[i].size());
  }
  std::vector<uint8_t> wctb((size_t)(nbits > 0 ? nbits : 1) * NR * NB);
  for (size_t o = 0; o < wctb.size() / NB; o++)
    for (int b = 0; b < NB; b++) wctb[o * NB + b] = (uint8_t)b;

  const size_t conf_size = 72 + 8 * (size_t)NB + 3 * sizeof(ea_hq) + sizeof(ea_xoshiro) + 8 + NB + NB * V / 8 + 4 * (size_t)NB;
  auto pack_data = [&](uint8_t *out, uint64_t sJ, uint64_t su, uint64_t sMC) {
    std::memset(out, 0, 72);
    const int32_t f[9] = {data.nbin, data.itcut, data.itmax, data.houfr, data.mesfr, data.ptfr, data.nbetas, data.flag, data.l};
    std::memcpy(out, f, 36);
    const uint64_t s[4] = {sJ, su, sMC, data.seed_C};
    std::memcpy(out + 40, s, 32);
  };
  std::vector<uint8_t> uu((size_t)NB * V), janus((size_t)NB * V / 8);

  // backup / read_conf (io.c:105-240, 854-868)
  if (data.flag == 0) {
    for (int i = 0; i < nbits; i++) {
      for (int r = 0; r < NR; r++) {
        const std::string name = dir_rep[i][r] + "/conf";
        struct stat st;
        stat(name.c_str(), &st);
        if ((size_t)st.st_size != conf_size) {
          create_error("There are only %d bytes in %s (must be %d)\n", (int)st.st_size, name.c_str(), (int)conf_size);
          print_and_exit("Problems reading confs\n");
        }
        FILE *f = fopen(name.c_str(), "rb");
        if (!f) { create_error("Problems opening %s\n", name.c_str()); print_and_exit("Problems reading confs\n"); }
        std::vector<uint8_t> raw(conf_size);
        if (fread(raw.data(), 1, conf_size, f) != conf_size) { create_error("Problems reading conf in %s\n", name.c_str()); print_and_exit("Problems reading confs\n"); }
        fclose(f);
        Data dc;
        int32_t h[9];
        std::memcpy(h, raw.data(), 36);
        dc.nbin = h[0]; dc.itcut = h[1]; dc.itmax = h[2]; dc.houfr = h[3]; dc.mesfr = h[4]; dc.ptfr = h[5];
        dc.nbetas = h[6]; dc.flag = h[7]; dc.l = h[8];
        uint64_t s4[4];
        std::memcpy(s4, raw.data() + 40, 32);
        check_data(dc);
        if (data.itmax != dc.itmax || data.houfr != dc.houfr || data.mesfr != dc.mesfr || data.ptfr != dc.ptfr) {
          create_error("Different data from input and %s\n", name.c_str()); print_and_exit("Problems reading confs\n");
        }
        if (seeds_J[i] != s4[0]) { create_error("Different seed_J generated and read in %s\n", name.c_str()); print_and_exit("Problems reading confs\n"); }
        if (seeds_u[i] != s4[1]) { create_error("Different seed_u generated and read in %s\n", name.c_str()); print_and_exit("Problems reading confs\n"); }
        if (data.seed_C != s4[3]) { create_error("Different data.seed_Cluster and read in %s\n", name.c_str()); print_and_exit("Problems reading confs\n"); }
        if (seeds_MC[r] != s4[2]) { create_error("Different seed_MC generated and read in %s\n", name.c_str()); print_and_exit("Problems reading confs\n"); }
        data.itcut = dc.itcut;
        stop(&data.nbin);
        size_t p = 72;
        for (int b = 0; b < NB; b++) {
          double v;
          std::memcpy(&v, raw.data() + p + 8 * b, 8);
          if (std::fabs(v - betas[b]) > 1e-12) {
            create_error("Different beta (ibeta=%d, %.12g != %.12g)\n", b, v, betas[b]);
            print_and_exit("Problems reading confs\n");
          }
        }
        p += 8 * NB;
        std::memcpy(&pt[(size_t)i * NR + r], raw.data() + p, sizeof(ea_hq)); p += sizeof(ea_hq);
        std::memcpy(&gen.prc[r], raw.data() + p, sizeof(ea_hq)); p += sizeof(ea_hq);
        std::memcpy(&gen.rc, raw.data() + p, sizeof(ea_hq)); p += sizeof(ea_hq);
        std::memcpy(&gen.xo[r], raw.data() + p, sizeof(ea_xoshiro)); p += sizeof(ea_xoshiro);
        std::memcpy(&gen.cuda_rng_offset, raw.data() + p, 8); p += 8;
        uint8_t *wc = &wctb[((size_t)i * NR + r) * NB];
        std::memcpy(wc, raw.data() + p, NB); p += NB;
        std::vector<int> seen(NB, 0);
        for (int b = 0; b < NB; b++)
          if (wc[b] >= NB || seen[wc[b]]++) {
            create_error("There is an error in the permutatuons in %s\n", name.c_str());
            print_and_exit("Problems reading confs\n");
          }
        for (size_t s = 0; s < (size_t)NB * V; s++) uu[s] = (raw[p + (s >> 3)] >> (s & 7)) & 1;  // io.c:263-280
        p += (size_t)NB * V / 8;
        for (int b = 0; b < NB; b++) {
          int32_t Eread, Esc;
          std::memcpy(&Eread, raw.data() + p + 4 * b, 4);
          ck(ea_host_scalar_energy(&geo, &uu[(size_t)wc[b] * V], J6[i].data(), &Esc), "scalar energy");
          if (Eread != Esc) {
            create_error("Energy read and calculate differ in ibit=%d ir=%d ibeta=%d:escalar=%d, read=%d\n", i, r, b, Esc, Eread);
            print_and_exit("Problems reading confs\n");
          }
        }
        ck(ea_host_pack_replica(&geo, uu.data(), r, ev[i].data(), od[i].data()), "packing");
      }
    }
    printf("Packing spins well done.\n");
    print_data(stdout, data);
    fflush(stdout);
    if (data.itcut >= data.nbin) {
      delete_running();
      create_error("There are %d iterations in %s\n", data.itcut, dir.c_str());
      print_and_exit("Problems in backup\n");
    }
  }
  if (write_seeds) {
    ignore_sigterm();
    FILE *f = fopen((dir + "/master_seeds.in").c_str(), "w");
    if (!f) { create_error("Impossible to open seed file to write\n"); print_and_exit("Problems writing seeds\n"); }
    fprintf(f, "%llu %llu %llu %llu\n", (unsigned long long)data.seed_J, (unsigned long long)data.seed_u,
            (unsigned long long)data.seed_MC, (unsigned long long)data.seed_C);
    fclose(f);
    handle_sigterm();
    for (int i = 0; i < nbits; i++) {
      ignore_sigterm();
      FILE *g = fopen((dirsample[i] + "/seeds.in").c_str(), "w");
      if (!g) { create_error("Impossible to open seed file to write\n"); print_and_exit("Problems writing seeds\n"); }
      fprintf(g, "%llu %llu", (unsigned long long)seeds_J[i], (unsigned long long)seeds_u[i]);
      for (int r = 0; r < NR; r++) fprintf(g, " %llu", (unsigned long long)seeds_MC[r]);
      fprintf(g, " %llu", (unsigned long long)data.seed_C);
      fprintf(g, " %d\n", countJ0[i]);
      fclose(g);
      handle_sigterm();
    }
  }
  stop(&data.nbin);
  if (nbits == 0) {
    ignore_sigterm();
    delete_running();
    printf("Simulation I=%d, nbits=%d finished at iteration %d\n", sample, nbits, data.itcut);
    return 0;
  }

  // device job
  ea_ctx *ctx = nullptr;
  ck(ea_create(&geo, device, &ctx), "ea_create");
  // without cluster moves no uniforms are drawn: the job keeps every SM
  if (!bld.cluster) ck(ea_set_rng_sms(ctx, 0), "SM split");
  ck(ea_set_temperatures(ctx, betas.data(), cum.data()), "temperatures");
  gen.seed_cluster = data.seed_C;
  ck(ea_set_generators(ctx, &gen, pt.data()), "generators");
  for (int i = 0; i < nbits; i++) {
    ck(ea_set_spins(ctx, i, ev[i].data(), od[i].data()), "spins");
    ck(ea_set_couplings(ctx, i, Jw[i].data()), "couplings");
  }
  ck(ea_set_permutations(ctx, wctb.data()), "permutations");
  // the restart counter omits houfr (main.cu:139)
  ck(ea_set_counter(ctx, 2LL * data.itcut * data.itmax * data.mesfr * data.ptfr, jobid), "counter");
  if (const char *e = getenv("EAGB_CLUSTER_EXACT")) ck(ea_set_cluster_rule(ctx, atoi(e) ? EA_CLUSTER_EXACT : EA_CLUSTER_REFERENCE), "cluster rule");
  const double spins_per_bin = (double)data.houfr * data.mesfr * data.ptfr * data.itmax * NB * (double)V * NR * nbits;
  measure_time(spins_per_bin);
  const ea_cadence cad{data.itmax, data.houfr, data.mesfr, data.ptfr, bld.cluster, 0};
  const size_t nsr = (size_t)nbits * NR;
  std::vector<double> avg(nsr * NB), acc(nsr * (NB - 1)), att(nsr * (NB - 1)), raw(nsr * (NB - 1));
  std::vector<uint8_t> hist(nsr * (size_t)maxit * NB);
  std::vector<int32_t> E(nsr * NB);
  std::vector<uint8_t> conf(conf_size);
  int ibin;
  for (ibin = data.itcut; ibin < data.nbin; ibin++) {
    renew_running();
    int32_t mx = 0;
    ck(ea_run_bin(ctx, &cad, avg.data(), hist.data(), &mx), "bin");
    measure_time(spins_per_bin);
    ignore_sigterm();
    // write_history (io.c:365-397)
    for (int i = 0; i < nbits; i++)
      for (int r = 0; r < NR; r++) {
        const std::string name = dir_rep[i][r] + "history_b.dat";
        struct stat st;
        const long actual = stat(name.c_str(), &st) == 0 ? (long)st.st_size : 0;
        const long predicted = (long)ibin * maxit * NB;
        FILE *f = fopen(name.c_str(), "a");
        if (!f) { create_error("Problems opening history_b.dat\n"); print_and_exit("Problems writing history\n"); }
        if (actual < predicted) { create_error("There are less data than expected in history_b.dat\n"); print_and_exit("Problems writing history\n"); }
        fwrite(&hist[(((size_t)i * NR + r) * maxit) * NB], 1, (size_t)maxit * NB, f);
        fclose(f);
      }
    for (auto &v : avg) v /= (double)data.itmax;
    ck(ea_get_pt_stats(ctx, acc.data(), att.data(), raw.data()), "pt stats");
    // write_measures (io.c:307-363)
    printf("Block = %d\n", ibin);
    for (int i = 0; i < nbits; i++) {
      printf("Sample = %d\n", list[i]);
      for (int r = 0; r < NR; r++) {
        printf("\t ir = %d: ", r);
        for (int b = 0; b < NB; b++) printf("E[%d]=%10.8g ", b, avg[((size_t)i * NR + r) * NB + b]);
        printf("\n");
      }
      fflush(stdout);
      for (int r = 0; r < NR; r++) {
        const size_t o = (size_t)i * NR + r;
        FILE *f = fopen((dir_rep[i][r] + "evol.txt").c_str(), "a");
        if (!f) { create_error("Problems opening evol.txt file\n"); print_and_exit("Problems writing measures\n"); }
        fprintf(f, "%d ", ibin);
        for (int b = 0; b < NB; b++) fprintf(f, "%14.10g ", avg[o * NB + b]);
        fprintf(f, "\n");
        fclose(f);
        f = fopen((dir_rep[i][r] + "aceptancePT.txt").c_str(), "a");
        if (!f) { create_error("Problems opening aceptance.txt file\n"); print_and_exit("Problems writing measures\n"); }
        fprintf(f, "#%d\n", ibin);
        for (int b = 0; b < NB - 1; b++) {
          const size_t k = o * (NB - 1) + b;
          fprintf(f, "%g %g %g %g\n", betas[b], acc[k] / att[k], raw[k] / att[k], att[k]);
        }
        fclose(f);
      }
    }
    // write_conf (io.c:17-103)
    ++data.itcut;
    ck(ea_measure_energy(ctx, E.data()), "energies");
    ck(ea_get_generators(ctx, &gen, pt.data()), "generator state");
    ck(ea_get_permutations(ctx, wctb.data(), nullptr), "permutations");
    for (int i = 0; i < nbits; i++) {
      ck(ea_get_spins(ctx, i, ev[i].data(), od[i].data()), "spins");
      for (int r = 0; r < NR; r++) {
        const size_t o = (size_t)i * NR + r;
        ck(ea_host_unpack_replica(&geo, ev[i].data(), od[i].data(), r, uu.data()), "unpacking");
        std::memset(janus.data(), 0, janus.size());
        for (size_t s = 0; s < (size_t)NB * V; s++) janus[s >> 3] |= (uint8_t)(uu[s] << (s & 7));
        uint8_t *p = conf.data();
        pack_data(p, seeds_J[i], seeds_u[i], seeds_MC[r]); p += 72;
        std::memcpy(p, betas.data(), 8 * NB); p += 8 * NB;
        std::memcpy(p, &pt[o], sizeof(ea_hq)); p += sizeof(ea_hq);
        std::memcpy(p, &gen.prc[r], sizeof(ea_hq)); p += sizeof(ea_hq);
        std::memcpy(p, &gen.rc, sizeof(ea_hq)); p += sizeof(ea_hq);
        std::memcpy(p, &gen.xo[r], sizeof(ea_xoshiro)); p += sizeof(ea_xoshiro);
        std::memcpy(p, &gen.cuda_rng_offset, 8); p += 8;
        std::memcpy(p, &wctb[o * NB], NB); p += NB;
        std::memcpy(p, janus.data(), janus.size()); p += janus.size();
        for (int b = 0; b < NB; b++) { std::memcpy(p, &E[o * NB + wctb[o * NB + b]], 4); p += 4; }
        char name[kMaxStr];
        snprintf(name, sizeof(name), "%s/conf.%06d", dir_rep[i][r].c_str(), data.itcut);
        write_file(name, conf.data(), conf.size());
        const std::string link_name = dir_rep[i][r] + "/conf";
        remove(link_name.c_str());
        if (link(name, link_name.c_str())) { create_error("Problems in hard-lin to %s\n", name); print_and_exit("Problems writing confs\n"); }
        struct stat st;
        stat(link_name.c_str(), &st);
        if (st.st_nlink != 2) { create_error("The number of hard-link %s is not 2\n", link_name.c_str()); print_and_exit("Problems writing confs\n"); }
        if ((size_t)st.st_size != conf_size) {
          create_error("There are only %d bytes in %s (must be %d)\n", (int)st.st_size, link_name.c_str(), (int)conf_size);
          print_and_exit("Problems writing confs\n");
        }
      }
    }
    stop(&data.nbin);
    handle_sigterm();
    if (check_time(max_time)) break;
  }
  ignore_sigterm();
  delete_running();
  printf("Simulation I=%d, nbits=%d finished at iteration %d\n", sample, nbits, ibin);
  fflush(stdout);
  ea_destroy(ctx);
  return 0;
}
