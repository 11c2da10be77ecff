// mmh_recon: the reference's driver program (mmh/main.f90) on the GB300
// library.  It reads the density file, optionally restarts from a checkpoint,
// runs the deformation iterations device-resident with main.f90's per-
// iteration diagnostics, writes the checkpoint and the output files -- all
// with the reference's file names and formats: raw stream files
// (access='stream'), Fortran column-major order, default real (4 bytes; 8
// with --real8).  Host code only; it calls the C ABI of include/mmh.h.
//
//   mmh_recon --ng N [--niter 300] [--workdir DIR/] [--z 0.000] [--inf den]
//             [--id _2] [--prefix .bin] [--fnu u512/] [--fndef def512/]
//             [--fndelta delta512/] [--fndisp disp512/] [--restart STEP]
//             [--no-def] [--no-gradient] [--no-density] [--no-checkpoint]
//             [--real8] [--precision fp64|mixed] [--schedule ref|tol|vcycle]
//             [--tol T] [--ps-dir DIR/] [--print-names]
//
// --ps-dir writes the power spectra the reference's Fisher script reads
// (calcfisherinfo.f90:26-27): ps48bins_<NG><id>.txt of the input density
// contrast and ps48bins_def_<NG><id>.txt of def, one "k P(k)" line per bin of
// 48, k in radians per cell (the units of defp2delta's |k|^2, so k^4 P_def is
// the reconstructed density's power, as calcfisherinfo.f90:66 forms it) and P
// in grid units (mean |DFT|^2 / n^3).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mmh.h"

namespace {

struct Opts {
  int ng = 0, niter = 300, restart = -1;
  std::string workdir = "./", z = "0.000", inf = "den", id = "_2", prefix = ".bin";
  std::string fnu = "u512/", fndef = "def512/", fndelta = "delta512/", fndisp = "disp512/";
  std::string psdir;
  bool flag_def = true, flag_gradient = true, flag_density = true, flag_check = true;
  bool real8 = false, print_names = false;
  int precision = MMH_FP64, schedule = MMH_SCHED_REF;
  double tol = 1e-8;
};

// i4.4 of the reference's write(gstring,'(i4.4)')
std::string i4(int v) {
  char b[32];
  std::snprintf(b, sizeof b, "%04d", v);
  return b;
}

// File names of main.f90:61, 122, 135-147, 166, 189-194 (restart) and 208-213.
struct Names {
  std::string input, def, psi[3], recon, restart_u, restart_def, check_u, check_def;
};
Names names_of(const Opts& o) {
  Names n;
  const std::string g = i4(o.ng);
  n.input = o.workdir + o.z + o.inf + g + o.id + o.prefix;
  n.def = o.workdir + o.fndef + o.z + "def" + o.id + g + o.prefix;
  const char* ax[3] = {"psix", "psiy", "psiz"};
  for (int a = 0; a < 3; ++a) n.psi[a] = o.workdir + o.fndisp + o.z + ax[a] + o.id + g + o.prefix;
  n.recon = o.workdir + o.fndelta + o.z + "recon" + o.id + g + o.prefix;
  const std::string rs = i4(o.restart < 0 ? 0 : o.restart), cs = i4(o.niter);
  n.restart_u = o.workdir + o.fnu + o.z + "restartu" + rs + "-" + o.id + g + o.prefix;
  n.restart_def = o.workdir + o.fndef + o.z + "restartdef" + rs + "-" + o.id + g + o.prefix;
  n.check_u = o.workdir + o.fnu + o.z + "restartu" + cs + "-" + o.id + g + o.prefix;
  n.check_def = o.workdir + o.fndef + o.z + "restartdef" + cs + "-" + o.id + g + o.prefix;
  return n;
}

int usage(const char* msg) {
  if (msg) std::fprintf(stderr, "mmh_recon: %s\n", msg);
  std::fprintf(stderr,
               "usage: mmh_recon --ng N [--niter K] [--workdir DIR/] [--z S] [--inf S] [--id S] [--prefix S]\n"
               "       [--fnu S] [--fndef S] [--fndelta S] [--fndisp S] [--restart STEP] [--no-def]\n"
               "       [--no-gradient] [--no-density] [--no-checkpoint] [--real8]\n"
               "       [--precision fp64|mixed] [--schedule ref|tol|vcycle] [--tol T] [--ps-dir DIR/]\n"
               "       [--print-names]\n");
  return 2;
}

bool parse(int argc, char** argv, Opts& o) {
  for (int a = 1; a < argc; ++a) {
    std::string k = argv[a];
    auto val = [&](std::string& dst) {
      if (a + 1 >= argc) return false;
      dst = argv[++a];
      return true;
    };
    std::string v;
    if (k == "--ng" && val(v)) o.ng = std::atoi(v.c_str());
    else if (k == "--niter" && val(v)) o.niter = std::atoi(v.c_str());
    else if (k == "--restart" && val(v)) o.restart = std::atoi(v.c_str());
    else if (k == "--workdir") { if (!val(o.workdir)) return false; }
    else if (k == "--z") { if (!val(o.z)) return false; }
    else if (k == "--inf") { if (!val(o.inf)) return false; }
    else if (k == "--id") { if (!val(o.id)) return false; }
    else if (k == "--prefix") { if (!val(o.prefix)) return false; }
    else if (k == "--fnu") { if (!val(o.fnu)) return false; }
    else if (k == "--fndef") { if (!val(o.fndef)) return false; }
    else if (k == "--fndelta") { if (!val(o.fndelta)) return false; }
    else if (k == "--fndisp") { if (!val(o.fndisp)) return false; }
    else if (k == "--ps-dir") { if (!val(o.psdir)) return false; }
    else if (k == "--no-def") o.flag_def = false;
    else if (k == "--no-gradient") o.flag_gradient = false;
    else if (k == "--no-density") o.flag_density = false;
    else if (k == "--no-checkpoint") o.flag_check = false;
    else if (k == "--real8") o.real8 = true;
    else if (k == "--print-names") o.print_names = true;
    else if (k == "--tol" && val(v)) o.tol = std::atof(v.c_str());
    else if (k == "--precision" && val(v)) {
      if (v == "fp64") o.precision = MMH_FP64;
      else if (v == "mixed") o.precision = MMH_MIXED;
      else return false;
    } else if (k == "--schedule" && val(v)) {
      if (v == "ref") o.schedule = MMH_SCHED_REF;
      else if (v == "tol") o.schedule = MMH_SCHED_TOL;
      else if (v == "vcycle") o.schedule = MMH_SCHED_VCYCLE;
      else return false;
    } else {
      return false;
    }
  }
  return o.ng > 0 && o.niter >= 0;
}

// A raw stream file of count reals (4 or 8 bytes) into / out of doubles.
bool read_reals(const std::string& fn, std::vector<double>& a, size_t count, bool real8) {
  FILE* f = std::fopen(fn.c_str(), "rb");
  if (!f) return false;
  a.assign(count, 0.0);
  bool ok;
  if (real8) {
    ok = std::fread(a.data(), sizeof(double), count, f) == count;
  } else {
    std::vector<float> t(count);
    ok = std::fread(t.data(), sizeof(float), count, f) == count;
    for (size_t q = 0; q < count; ++q) a[q] = (double)t[q];
  }
  std::fclose(f);
  return ok;
}
bool write_reals(const std::string& fn, const double* a, size_t count, bool real8) {
  FILE* f = std::fopen(fn.c_str(), "wb");
  if (!f) return false;
  bool ok;
  if (real8) {
    ok = std::fwrite(a, sizeof(double), count, f) == count;
  } else {
    std::vector<float> t(a, a + count);
    ok = std::fwrite(t.data(), sizeof(float), count, f) == count;
  }
  return std::fclose(f) == 0 && ok;
}

// sum(real(x,8)) / n^3 and sqrt(sum(real((x-c)**2,8)) / n^3), as main.f90
// prints them (sequential FP64 sums)
double mean_of(const std::vector<double>& a) {
  double s = 0.0;
  for (double x : a) s += x;
  return s / (double)a.size();
}
double rms_about(const std::vector<double>& a, double c) {
  double s = 0.0;
  for (double x : a) s += (x - c) * (x - c);
  return std::sqrt(s / (double)a.size());
}

// The 48-bin power spectrum of a field in the Fisher script's layout.
bool write_spectrum(mmh_ctx* ctx, const std::string& fn, const double* a, int n) {
  const int nb = 48;
  double k[nb], p[nb];
  if (mmh_power_spectrum_f64(ctx, a, nullptr, nb, k, p, nullptr) != MMH_OK) return false;
  FILE* f = std::fopen(fn.c_str(), "w");
  if (!f) return false;
  const double unit = 2.0 * 3.14159265358979323846 / n;
  for (int q = 0; q < nb; ++q) std::fprintf(f, "%.16e %.16e\n", k[q] * unit, p[q]);
  return std::fclose(f) == 0;
}

int write_failed() {
  std::fprintf(stderr, "mmh_recon: write failed\n");
  return 1;
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

#define TRY(call, what)                                                        \
  do {                                                                         \
    int rc_ = (call);                                                          \
    if (rc_ != MMH_OK && rc_ != MMH_ERR_DIVERGED) {                            \
      std::fprintf(stderr, "mmh_recon: %s: %s\n", what, mmh_strerror(rc_));    \
      return 1;                                                                \
    }                                                                          \
  } while (0)

}  // namespace

int main(int argc, char** argv) {
  Opts o;
  if (!parse(argc, argv, o)) return usage(argc > 1 ? "bad arguments" : nullptr);
  const Names fn = names_of(o);
  if (o.print_names) {
    std::printf("input %s\nrestart_u %s\nrestart_def %s\ncheckpoint_u %s\ncheckpoint_def %s\ndef %s\n"
                "psix %s\npsiy %s\npsiz %s\nrecon %s\n",
                fn.input.c_str(), fn.restart_u.c_str(), fn.restart_def.c_str(), fn.check_u.c_str(),
                fn.check_def.c_str(), fn.def.c_str(), fn.psi[0].c_str(), fn.psi[1].c_str(), fn.psi[2].c_str(),
                fn.recon.c_str());
    return 0;
  }
  const int n = o.ng;
  const size_t n3 = (size_t)n * n * n;
  std::printf(" grid: %d\n \n BEGIN\n", n);
  // input density (main.f90:58-80)
  double t1 = now();
  std::vector<double> rho, def(n3, 0.0);
  std::printf(" reading: %s\n", fn.input.c_str());
  if (!read_reals(fn.input, rho, n3, o.real8)) {
    std::fprintf(stderr, "mmh_recon: cannot read %zu reals from %s\n", n3, fn.input.c_str());
    return 1;
  }
  std::printf(" time consumed for reading: %g seconds\n \n u:\n", now() - t1);
  const double umean = mean_of(rho);
  if (std::fabs(umean - 1.0) > 1.e-5) {
    std::printf(" umean should be zero, program ended\n");
    return 1;
  }
  std::printf(" u mean= %.7g\n u sigma= %.7g\n \n BEGIN MULTIGRID\n", umean, rms_about(rho, 1.0));
  std::vector<double> contrast;
  if (!o.psdir.empty()) {
    contrast.resize(n3);
    for (size_t q = 0; q < n3; ++q) contrast[q] = rho[q] - 1.0;
  }
  int begin = 1;
  if (o.restart >= 0) {
    // readrestart (main.f90:184-200)
    begin = o.restart + 1;
    std::printf(" \n RESTART!\n reading: %s\n", fn.restart_u.c_str());
    if (!read_reals(fn.restart_u, rho, n3, o.real8)) {
      std::fprintf(stderr, "mmh_recon: cannot read %s\n", fn.restart_u.c_str());
      return 1;
    }
    std::printf(" reading: %s\n", fn.restart_def.c_str());
    if (!read_reals(fn.restart_def, def, n3, o.real8)) {
      std::fprintf(stderr, "mmh_recon: cannot read %s\n", fn.restart_def.c_str());
      return 1;
    }
    std::printf(" def sigma= %.7g\n u sigma= %.7g\n", rms_about(def, 0.0), rms_about(rho, 1.0));
  }
  mmh_config cfg;
  mmh_config_default(&cfg, n);
  cfg.precision = o.precision;
  cfg.schedule = o.schedule;
  cfg.tol = o.tol;
  mmh_ctx* ctx = nullptr;
  TRY(mmh_create(&ctx, &cfg), "mmh_create");
  TRY(mmh_load_f64(ctx, def.data(), rho.data(), 1), "mmh_load_f64");
  // the deformation iterations (main.f90:90-110)
  for (int iter = begin; iter <= o.niter; ++iter) {
    const double w1 = now();
    std::printf(" \n iter= %d\n", iter);
    mmh_diag d;
    TRY(mmh_iterate(ctx, 1, &d), "mmh_iterate");
    mmh_stats st;
    TRY(mmh_state_stats(ctx, &st), "mmh_state_stats");
    std::printf(" CALCDEFP\n defp sigma= %.7g\n DEF+DEFP\n def sigma= %.7g\n RELAXING\n u sigma= %.7g\n"
                " u min max= %.7g %.7g\n u < 0 : %lld\n real time consumed for one iteration: %g seconds\n",
                st.defp_sigma, st.def_sigma, st.rho_sigma, st.rho_min, st.rho_max, st.rho_negative, now() - w1);
    std::fflush(stdout);
  }
  std::vector<double> u(n3);
  TRY(mmh_store_f64(ctx, def.data(), u.data(), 1), "mmh_store_f64");
  if (o.flag_check) {
    // checkpoint (main.f90:202-216)
    std::printf(" \n CHECKPOINT!\n writing: %s\n", fn.check_u.c_str());
    if (!write_reals(fn.check_u, u.data(), n3, o.real8)) return write_failed();
    std::printf(" writing: %s\n", fn.check_def.c_str());
    if (!write_reals(fn.check_def, def.data(), n3, o.real8)) return write_failed();
  }
  std::printf(" END MULTIGRID\n \n def:\n avg= %.7g\n sigma= %.7g\n", mean_of(def), rms_about(def, 0.0));
  // outputs (main.f90:120-179)
  if (o.flag_def) {
    std::printf(" writing: %s\n", fn.def.c_str());
    if (!write_reals(fn.def, def.data(), n3, o.real8)) return write_failed();
  }
  if (o.flag_gradient || o.flag_density) {
    std::vector<double> grad(o.flag_gradient ? 3 * n3 : 0), delta(o.flag_density ? n3 : 0);
    t1 = now();
    TRY(mmh_outputs_f64(ctx, o.flag_gradient ? grad.data() : nullptr, o.flag_density ? delta.data() : nullptr),
        "mmh_outputs_f64");
    if (o.flag_gradient) {
      for (int a = 0; a < 3; ++a) {
        std::printf(" writing: %s\n", fn.psi[a].c_str());
        if (!write_reals(fn.psi[a], grad.data() + a * n3, n3, o.real8))
          return write_failed();
      }
      std::printf(" time consumed for defp2phi: %g seconds\n", now() - t1);
    }
    if (o.flag_density) {
      std::printf(" writing: %s\n", fn.recon.c_str());
      if (!write_reals(fn.recon, delta.data(), n3, o.real8)) return write_failed();
      std::printf(" \n time consumed for defp2delta: %g seconds\n delta:\n avg= %.7g\n sigma= %.7g\n", now() - t1,
                  mean_of(delta), rms_about(delta, 0.0));
    }
  }
  if (!o.psdir.empty()) {
    const std::string tag = std::to_string(n) + o.id + ".txt";
    const std::string f1 = o.psdir + "ps48bins_" + tag, f2 = o.psdir + "ps48bins_def_" + tag;
    std::printf(" writing: %s\n writing: %s\n", f1.c_str(), f2.c_str());
    if (!write_spectrum(ctx, f1, contrast.data(), n) || !write_spectrum(ctx, f2, def.data(), n)) return write_failed();
  }
  mmh_destroy(ctx);
  return 0;
}
