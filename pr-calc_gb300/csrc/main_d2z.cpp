// main_d2z.cpp — drop-in `delta2zreion` executable on the GB300 path.
//
// Same command line (commandline_d2z.C:6-126), parameter file grammar and
// -usedvalues echo (io_d2z.C:16-162), raw float32 grids (io_d2z.C:164-245,
// parallel_io.C:11-43) and printed diagnostics as the reference's main
// (main_d2z.C:15-109); the FFTW-MPI transforms and the delta2zreion() loop are
// replaced by one call through the C ABI (include/prc_d2z.h).  One process,
// one GPU: there is no MPI and the slab decomposition is gone.
#include <ctype.h>
#include <errno.h>
#include <fcntl.h>
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <string>
#include <vector>

#include "../../include/prc_d2z.h"

namespace {

struct Parameter {
  float Omegam = 0, Omegab = 0, Omegal = 0, h = 0, ns = 0, sigma8 = 0, w = 0;
  float BoxSize = 0, zInit = 0, Rmin = 0;
  int N = 0, Nscales = 0;
  char DeltaFile[256] = "";
  int RecordBubbleSizes = 0;
};

struct ClParameter {
  float Rmax = 256, zeta = 10, M_min = 1e8;
  int verbose = 0, everbose = 0, lean = 0;
  char Paramfile[256] = "", Basename[256] = "output/output";
};

Parameter P;
ClParameter CL;

void usage() {
  printf("\n usage: d2z <parameterfile> [options]\n");
  printf("\n OPTIONS:\n");
  printf("\n   -h show this message");
  printf("\n   -f <File base name> [default = 'output'; all output files will be prepended");
  printf("\n      with this string and placed in a directory called output in the working");
  printf("\n      directory (e.g. output/output.history, output/output.zreion, etc)]");
  printf("\n   -r <Rmfp> [default = 256; this is the mean free path in units of Mpc/h]");
  printf("\n   -m <Mmin> [default = 1e8; this is the minimum halo mass");
  printf("\n      capable of hosting ionizing sources, in Msun]");
  printf("\n   -z <zeta> [default =  10; this is the efficiency of halos in ionizing");
  printf("\n      their surroundings -- i.e. zeta = M_HII / Mhalo * rho_matter / rho_hydrogen]");
  printf("\n   -l lean mode (accepted; the GPU path keeps the spectrum resident, so it changes nothing)");
  printf("\n   -v switch on verbose mode to print stdout to terminal instead of .stdout file [default = OFF]");
  printf("\n   -e switch on verbose mode to print stderr to terminal instead of .stderr file [default = OFF]");
  printf("\n\n");
  exit(0);
}

// commandline_d2z.C:33-126
void CommandLine(int argc, char* argv[]) {
  opterr = 0;
  if (argc < 2) usage();
  snprintf(CL.Paramfile, sizeof(CL.Paramfile), "%s", argv[1]);
  snprintf(CL.Basename, sizeof(CL.Basename), "output/output");
  mkdir("output", 0777);
  int c;
  while ((c = getopt(argc - 1, &argv[1], "hvelf:r:m:z:")) != -1) {
    switch (c) {
      case 'h': usage(); break;
      case 'f': snprintf(CL.Basename, sizeof(CL.Basename), "output/%s", optarg); break;
      case 'r': CL.Rmax = (float)atof(optarg); break;
      case 'm': CL.M_min = (float)atof(optarg); break;
      case 'z': CL.zeta = (float)atof(optarg); break;
      case 'v': CL.verbose = 1; break;
      case 'e': CL.everbose = 1; break;
      case 'l': CL.lean = 1; break;
      case '?':
        if (optopt == 'r' || optopt == 'f' || optopt == 'm' || optopt == 'z')
          fprintf(stderr, "\n Option -%c requires an argument.\n", optopt);
        else if (isprint(optopt))
          fprintf(stderr, "\n Unknown option `-%c'.\n", optopt);
        else
          fprintf(stderr, "Unknown option character `\\x%x'.\n", optopt);
        usage();
        return;
      default: usage();
    }
  }
  if (CL.verbose == 0) {
    std::string f = std::string(CL.Basename) + ".stdout";
    if (!freopen(f.c_str(), "w", stdout)) fprintf(stderr, "cannot open %s\n", f.c_str());
  }
  if (CL.everbose == 0) {
    std::string f = std::string(CL.Basename) + ".stderr";
    if (!freopen(f.c_str(), "w", stderr)) fprintf(stdout, "cannot open %s\n", f.c_str());
  }
  setvbuf(stdout, NULL, _IONBF, 0);
  setvbuf(stderr, NULL, _IONBF, 0);
  printf("\n Command line: %s %s", argv[0], argv[argc - 1]);
  for (int i = 1; i < argc - 1; i++) printf(" %s", argv[i]);
  printf("\n");
}

// io_d2z.C:16-162: tag/value file, '%'/'#' comments, each tag once, echo to
// <paramfile>-usedvalues.  Returns 0 when the file could not be opened.
int ReadParameterFile() {
  enum { FLOAT, STRING, INT };
  struct Tag {
    const char* name;
    void* addr;
    int type;
    bool used;
  } tags[] = {{"Omegam", &P.Omegam, FLOAT, false}, {"Omegab", &P.Omegab, FLOAT, false},
              {"Omegal", &P.Omegal, FLOAT, false}, {"h", &P.h, FLOAT, false},
              {"ns", &P.ns, FLOAT, false},         {"sigma8", &P.sigma8, FLOAT, false},
              {"w", &P.w, FLOAT, false},           {"BoxSize", &P.BoxSize, FLOAT, false},
              {"zInit", &P.zInit, FLOAT, false},   {"Rmin", &P.Rmin, FLOAT, false},
              {"N", &P.N, INT, false},             {"Nscales", &P.Nscales, INT, false},
              {"DeltaFile", P.DeltaFile, STRING, false},
              {"RecordBubbleSizes", &P.RecordBubbleSizes, INT, false}};
  P.RecordBubbleSizes = 0;
  FILE* fd = fopen(CL.Paramfile, "r");
  if (!fd) {
    printf("\nParameter file %s not found.\n\n", CL.Paramfile);
    return 0;
  }
  std::string echo = std::string(CL.Paramfile) + "-usedvalues";
  FILE* fdout = fopen(echo.c_str(), "w");
  if (!fdout) {
    printf("error opening file '%s' \n", echo.c_str());
    fclose(fd);
    return 0;
  }
  char buf[200], b1[200], b2[200], b3[400];
  while (fgets(buf, sizeof(buf), fd)) {
    if (sscanf(buf, "%199s%199s%399s", b1, b2, b3) < 2) continue;
    if (b1[0] == '%' || b1[0] == '#') continue;
    Tag* t = nullptr;
    for (auto& q : tags)
      if (!q.used && strcmp(b1, q.name) == 0) {
        t = &q;
        break;
      }
    if (!t) {
      fprintf(stdout, "Error in %s: Tag '%s' not allowed or multiple defined.\n", CL.Paramfile, b1);
      continue;
    }
    t->used = true;
    switch (t->type) {
      case FLOAT:
        *(float*)t->addr = (float)atof(b2);
        fprintf(fdout, "%-35s%f\n", b1, *(float*)t->addr);
        break;
      case STRING:
        snprintf((char*)t->addr, 256, "%s", b2);
        fprintf(fdout, "%-35s%s\n", b1, b2);
        break;
      case INT:
        *(int*)t->addr = atoi(b2);
        fprintf(fdout, "%-35s%d\n", b1, *(int*)t->addr);
        break;
    }
  }
  fclose(fd);
  fclose(fdout);
  printf("\n Parameter file read...");
  return 1;
}

// parallel_io.C:11-43 semantics: pread/pwrite of whole byte ranges
bool read_all(const char* fname, void* buf, size_t size) {
  int fd = open(fname, O_RDONLY);
  if (fd < 0) return false;
  size_t done = 0;
  while (done < size) {
    ssize_t r = pread(fd, (char*)buf + done, size - done, (off_t)done);
    if (r <= 0) break;
    done += (size_t)r;
  }
  close(fd);
  return done == size;
}

bool write_all(const char* fname, const void* buf, size_t size) {
  int fd = open(fname, O_RDWR | O_CREAT, S_IRUSR | S_IWUSR);
  if (fd < 0) return false;
  size_t done = 0;
  while (done < size) {
    ssize_t r = pwrite(fd, (const char*)buf + done, size - done, (off_t)done);
    if (r <= 0) break;
    done += (size_t)r;
  }
  close(fd);
  return done == size;
}

int fail(const char* what, int st) {
  fprintf(stderr, "\n delta2zreion: %s failed (%d): %s\n", what, st, prc_last_error());
  printf("\n delta2zreion: %s failed (%d): %s\n", what, st, prc_last_error());
  return 1;
}

}  // namespace

int main(int argc, char* argv[]) {
  CommandLine(argc, argv);
  if (!ReadParameterFile()) return 1;
  const int N = P.N;
  const long long n3 = (long long)N * N * N;
  if (!prc_d2z_supported(N)) {
    printf("\n grid size N=%d has no GPU FFT plan\n", N);
    return 1;
  }
  // main_d2z.C:52-55 / io_d2z.C:164-207
  std::vector<float> delta((size_t)n3);
  if (!read_all(P.DeltaFile, delta.data(), sizeof(float) * n3)) {
    printf("\n cannot read %lld floats from %s\n", n3, P.DeltaFile);
    return 1;
  }
  {
    double mean = 0, sigma = 0;
    for (long long i = 0; i < n3; ++i) {
      mean += delta[i];
      sigma += (double)delta[i] * delta[i];
    }
    mean /= pow((float)N, 3);
    sigma /= pow((float)N, 3);
    sigma = sqrt(sigma);
    printf("\n Input data read, mean = %le sigma = %le", mean, sigma);
  }
  // host tables (main_d2z.C:57-64, delta2zreion_d2z.C:14-38)
  prc_params pp;
  pp.Omegam = P.Omegam; pp.Omegab = P.Omegab; pp.Omegal = P.Omegal; pp.h = P.h; pp.ns = P.ns;
  pp.sigma8 = P.sigma8; pp.w = P.w; pp.BoxSize = P.BoxSize; pp.zInit = P.zInit; pp.Rmin = P.Rmin;
  pp.N = N; pp.Nscales = P.Nscales; pp.Rmax = CL.Rmax; pp.zeta = CL.zeta; pp.M_min = CL.M_min;
  std::vector<double> R(P.Nscales), B(P.Nscales);
  std::vector<float> sig(P.Nscales);
  prc_tables tb;
  memset(&tb, 0, sizeof(tb));
  tb.radii_mpc = R.data();
  tb.sigma_r = sig.data();
  tb.barrier_b = B.data();
  int st = prc_compute_tables(&pp, &tb);
  if (st != PRC_OK) return fail("prc_compute_tables", st);

  prc_d2z_desc d;
  memset(&d, 0, sizeof(d));
  d.N = N;
  d.n_radii = P.Nscales;
  d.box_mpc = (double)(P.BoxSize / P.h);
  d.radii_mpc = R.data();
  d.barrier_b = B.data();
  d.barrier_a = tb.barrier_a;
  d.growth_init = tb.DInit;
  d.flags = PRC_FLAG_SIGMA_GRID | (P.RecordBubbleSizes == 1 ? PRC_FLAG_ARGMAX : 0);
  prc_d2z_ctx* ctx = nullptr;
  if ((st = prc_d2z_create(&d, &ctx)) != PRC_OK) return fail("prc_d2z_create", st);
  printf("\n Arrays allocated...");

  std::vector<float> zreion((size_t)n3);
  std::vector<uint8_t> argmax;
  if (P.RecordBubbleSizes == 1) argmax.resize((size_t)n3);
  std::vector<double> sgrid(P.Nscales);
  st = prc_d2z_forward(ctx, delta.data(), 0, zreion.data(), argmax.empty() ? nullptr : argmax.data(), 0,
                       sgrid.data());
  if (st != PRC_OK) return fail("prc_d2z_forward", st);

  // delta2zreion_d2z.C:46-52,102-103: the per-scale table
  const float Rinitial = (P.BoxSize / P.h) * P.Rmin / N;
  const float Rfinal = CL.Rmax / P.h;
  printf("\n");
  printf("\n Nscales = %2d    Rmin=%5.3f", P.Nscales, Rinitial * P.h);
  printf("\n                 Rmax=%5.3f\n", Rfinal * P.h);
  printf("\n      Scale       R [Mpc/h]        sigma(R)      sigma_grid");
  printf("\n ==========================================================\n");
  for (int r = 0; r < P.Nscales; ++r)
    printf("\n %10d %15.3f %15.3f %15.3f", r, (float)R[r] * P.h, sig[r], (float)sgrid[r]);
  printf("\n");
  float ms[3];
  if (prc_d2z_last_timing(ctx, ms) == PRC_OK)
    printf("\n GPU time: forward R2C %.3f ms, %d radii %.3f ms", ms[0], P.Nscales, ms[1]);

  // GetHistory (main_d2z.C:76, bubblehistory_d2z.C:5-43)
  std::vector<float> hist(PRC_NHISTORY), histz(PRC_NHISTORY);
  if ((st = prc_d2z_history(ctx, zreion.data(), 0, nullptr, hist.data(), histz.data())) != PRC_OK)
    return fail("prc_d2z_history", st);

  // GetBubbleMFP (main_d2z.C:79) with WriteMFP / WriteMFPPDF (io_d2z.C:343-402)
  prc_mfp_setup mset;
  mset.N = N;
  mset.box_mpc = P.BoxSize / P.h;
  mset.n_x = PRC_NX_MFP;
  mset.n_skewers = PRC_NSKEWERS;
  std::vector<float> mfp(PRC_NX_MFP), mfp_x(PRC_NX_MFP), dfdmfp((size_t)PRC_NMFP * PRC_NX_MFP);
  if ((st = prc_d2z_bubble_mfp(ctx, &mset, zreion.data(), hist.data(), mfp.data(), mfp_x.data(), dfdmfp.data())) !=
      PRC_OK)
    return fail("prc_d2z_bubble_mfp", st);
  printf("\n Writing bubble mfp...");
  {
    std::string f = std::string(CL.Basename) + ".mfp";
    FILE* fd = fopen(f.c_str(), "w");
    if (!fd) {
      printf("\n File %s could not be opened\n\n", f.c_str());
      return 1;
    }
    for (int i = 0; i < PRC_NX_MFP; i++) fprintf(fd, "%f %f\n", mfp_x[i], mfp[i]);
    fclose(fd);
  }
  printf("\n Writing bubble mfp...");
  {
    std::string f = std::string(CL.Basename) + ".mfppdf";
    FILE* fd = fopen(f.c_str(), "wb");
    if (!fd) {
      printf("\n File %s could not be opened\n\n", f.c_str());
      return 1;
    }
    const float box = P.BoxSize / P.h, cell = box / N;
    const int h1[2] = {PRC_NX_MFP, PRC_NMFP};
    const float h2[4] = {0.01f, 0.999f, (float)log10(1 * cell), (float)log10(1.0 * box)};
    fwrite(h1, sizeof(int), 2, fd);
    fwrite(h2, sizeof(float), 4, fd);
    fwrite(dfdmfp.data(), sizeof(float), dfdmfp.size(), fd);
    fclose(fd);
  }

  // GetCHistory (main_d2z.C:84) and CorrectHistory (:87); both need the
  // collapsed-fraction table fcoll_table.tab in the working directory
  prc_f2f_table fct;
  if ((st = prc_f2f_load("fcoll_table.tab", &fct)) != PRC_OK) return fail("reading fcoll_table.tab", st);
  std::vector<float> chist(PRC_NCHISTORY), zvz(PRC_NHISTORY);
  if ((st = prc_chistory(&fct, mfp.data(), PRC_NX_MFP, CL.Rmax, CL.zeta, chist.data())) != PRC_OK)
    return fail("prc_chistory", st);
  if ((st = prc_zvz(hist.data(), chist.data(), zvz.data())) != PRC_OK) return fail("prc_zvz", st);
  if ((st = prc_d2z_correct(ctx, zvz.data(), zreion.data(), 0)) != PRC_OK) return fail("prc_d2z_correct", st);

  // WriteZreionFile (main_d2z.C:90, io_d2z.C:209-245)
  printf("\n Writing reionization redshifts...");
  std::string zname = std::string(CL.Basename) + ".zreion";
  if (!write_all(zname.c_str(), zreion.data(), sizeof(float) * n3)) {
    printf("\n cannot write %s\n", zname.c_str());
    return 1;
  }
  printf("\n Reionization redshifts written...");
  if (P.RecordBubbleSizes == 1) {
    // the .rbubble writer (io_d2z.C:248-282; its call is commented out at
    // main_d2z.C:95): R of the winning scale, 0 where none won
    std::vector<float> rb((size_t)n3);
    for (long long i = 0; i < n3; ++i) rb[i] = argmax[i] == PRC_ARGMAX_NONE ? 0.f : (float)R[argmax[i]];
    std::string rname = std::string(CL.Basename) + ".rbubble";
    if (!write_all(rname.c_str(), rb.data(), sizeof(float) * n3)) {
      printf("\n cannot write %s\n", rname.c_str());
      return 1;
    }
    printf("\n Bubble sizes written...");
  }
  // GetHistory of the corrected field, tau (main_d2z.C:97-98), WriteHistory (:101)
  if ((st = prc_d2z_history(ctx, zreion.data(), 0, nullptr, hist.data(), histz.data())) != PRC_OK)
    return fail("prc_d2z_history", st);
  const float tau = prc_tau(histz.data(), hist.data(), PRC_NHISTORY, P.Omegam, P.Omegab, P.h);
  printf("\n\n tau = %f", tau);
  printf("\n Writing ionization history...");
  std::string hname = std::string(CL.Basename) + ".history";
  FILE* fh = fopen(hname.c_str(), "w");
  if (!fh) {
    printf("\n File %s could not be opened\n\n", hname.c_str());
    return 1;
  }
  for (int i = 0; i < PRC_NHISTORY; i++)
    fprintf(fh, "%e %e %e %e\n", histz[i], hist[i], prc_f2f_eval(&fct, histz[i]),
            prc_fcoll(histz[i], P.zInit, P.Omegam, P.Omegal, P.w, tb.sigma_min));
  fclose(fh);
  prc_f2f_free(&fct);
  prc_d2z_destroy(ctx);
  printf("\n\n");
  return 0;
}
