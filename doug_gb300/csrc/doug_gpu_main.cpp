// doug_gpu / doug_geom_gpu: the command-line drivers of the GB300 solve path
// (doug_aggr's setup, aggr.F90, and doug_geom's, geom.F90; the second is this
// file built with DG_DRIVER_GEOM), with the flags of the reference's
// executables (util_parseArgs, DOUG_utils.F90:485-566):
//   -f file.name    control file (default DOUG.dat)
//   -q [file.name]  quiet: the driver's messages go to file.name (default log.DOUG)
//   -p [prefix]     profile: phase times to prefix.00 (default prof)
//   -i              list the supported control words and exit
//   -v              print the version and exit
//   -h              print the usage and exit
// It reads the control file and its input files, builds the setup, solves
// with the stored right-hand side and writes solution_file when the control
// file names one, reporting as doug_aggr does (aggr.F90:246-258).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/doug_gpu.h"

namespace {

// the reference's control words (controls.F90:159-246), then the words only
// this build reads
const char *kReferenceWords[] = {
    "assembled_mtx_file", "assembled_mtx_format", "assembled_rhs_file", "assembled_rhs_format", "info_file",
    "elemmat_rhs_file", "freedom_lists_file", "coords_file", "freemap_file", "solution_format", "solution_file",
    "freedom_mask_file", "start_vec_type", "start_vec_file", "dump_matrix_only", "dump_matrix_file", "maxcie",
    "maxnd", "cutbal", "center_type", "hanging_nodes", "mass_matrix_file", "matrix_file", "rhs_file", "xyz_file",
    "solver", "method", "fine_method", "num_iters", "grid_size", "coarse_method", "levels", "num_subdomains",
    "overlap", "smoothers", "radius1", "radius2", "minasize1", "minasize2", "maxasize1", "maxasize2", "debug",
    "verbose", "plotting", "strong1", "strong2", "solve_tolerance", "input_type", "number_of_blocks",
    "matrix_type", "initial_guess", "symmstruct", "symmnumeric", "solve_maxiters", "interpolation_type",
    "submeth", "gmres_max_it", "gmrestarts"};
const char *kExtensionWords[] = {"precision", "replace_every", "omega", "nd_leaf", "profile", "reuse_factors",
                                 "elemental_matvec", "panel_rows", "fwd_task_kb", "lean_task_kb",
                                 "thin_level_fronts", "solve_schedule", "solve_pdl", "factor_overlap", "executable"};
#ifdef DG_DRIVER_GEOM
const char *kName = "doug_geom_gpu";
#else
const char *kName = "doug_gpu";
#endif

void usage(FILE *o) {
  fprintf(o, " Usage: \n");
  fprintf(o, " ./%s [[-f file.name] [-q [file.name]] [-p [file.prefix]] or [-i][-v][-h]]\n", kName);
  fprintf(o, "                 : w/o any parameter assumes control file is DOUG.dat\n");
  fprintf(o, " -f file.name    : specifies DOUG control file name\n");
  fprintf(o, " -q [file.name]  : quiet mode - the driver logs to log.DOUG or to file.name\n");
  fprintf(o, " -i              : prints out control file parameters and exits\n");
  fprintf(o, " -v              : prints the version and exits\n");
  fprintf(o, " -h              : prints this message and exits\n");
  fprintf(o, " -p [file.prefix]: phase times to file.prefix.00 (default prof.00)\n");
}

bool is_value(int i, int argc, char **argv) { return i < argc && argv[i][0] != '\0' && argv[i][0] != '-'; }

}  // namespace

int main(int argc, char **argv) {
  std::string ctl = "DOUG.dat", logname, profname;
  bool quiet = false, prof = false, ctl_set = false;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    if (a == "-f") {
      if (!is_value(i + 1, argc, argv)) {
        fprintf(stdout, " DOUG error: no control file given\n");
        usage(stdout);
        return 1;
      }
      ctl = argv[++i];
      ctl_set = true;
    } else if (a == "-q") {
      quiet = true;
      logname = is_value(i + 1, argc, argv) ? argv[++i] : "log.DOUG";
    } else if (a == "-p") {
      prof = true;
      profname = std::string(is_value(i + 1, argc, argv) ? argv[++i] : "prof") + ".00";
    } else if (a == "-i") {
      printf(" List of currently supported control parameters:\n");
      for (const char *w : kReferenceWords) printf(" %s\n", w);
      for (const char *w : kExtensionWords) printf(" %s\n", w);
      return 0;
    } else if (a == "-v") {
      printf(" DOUG version : GB300 solve path (doug_gb300)\n");
      return 0;
    } else if (a == "-h") {
      usage(stdout);
      return 0;
    } else {
      usage(stdout);
      fprintf(stdout, " DOUG error: Unrecognised command line parameter: %s\n", a.c_str());
      return 1;
    }
  }
  FILE *out = stdout;
  if (quiet) {
    out = fopen(logname.c_str(), "w");
    if (!out) {
      fprintf(stderr, " DOUG error: cannot open %s\n", logname.c_str());
      return 1;
    }
  }
  if (argc > 1 && !ctl_set) {
    fprintf(out, " Warning: No -f option specified.\n");
    fprintf(out, "          Give -h argument to see how to invoke the program.\n");
    fprintf(out, "          Assuming DOUG control file: %s\n", ctl.c_str());
  }
  dg_handle *h = nullptr;
  int rc = 1;
  auto fail = [&](const char *what, dg_status st) {
    fprintf(out, " DOUG error: %s: %s\n", what, h ? dg_last_error(h) : "");
    return st == DG_OK ? 1 : (int)st;
  };
  if (dg_create(&h) != DG_OK) {
    fprintf(out, " DOUG error: dg_create failed\n");
    return 1;
  }
  if (prof) dg_set_option(h, "profile", "1");  // phase times (event pairs, no iteration graph)
#ifdef DG_DRIVER_GEOM
  dg_set_option(h, "executable", "geom");  // the first value of a word wins: the control file cannot undo it
#endif
  dg_status st = dg_load_ctl(h, ctl.c_str());
  if (st != DG_OK) {
    rc = fail("control file", st);
  } else if ((st = dg_setup(h)) != DG_OK) {
    rc = fail("setup", st);
  } else {
    int n = 0, nf = 0, nc = 0, nsd = 0, rn = 0, an = 0;
    long long tot = 0;
    dg_get_sizes(h, &n, &nf, &nc, &nsd, &tot, &rn, &an);
    fprintf(out, " # coarse aggregates: %d\n", nc);
    fprintf(out, " calling pcg_weigs\n");
    std::vector<double> x((size_t)n);
    dg_stats s{};
    st = dg_solve(h, nullptr, x.data(), &s);
    if (st != DG_OK && st != DG_NOT_CONVERGED) {
      rc = fail("solve", st);
    } else {
      fprintf(out, " #it: %d  Cond#: %.6e\n", s.iterations, s.cond_num);
      fprintf(out, " true relative residual: %.6e%s\n", s.true_rel_residual,
              st == DG_NOT_CONVERGED ? "  (maximum iterations reached)" : "");
      const double t = s.t_setup_s + s.t_total_s;
      fprintf(out, " time spent in pcg(): %.6f\n", t);
      fprintf(out, "     ...of which setup: %.6f\n", s.t_setup_s + s.t_factor_s);
      fprintf(out, "        ...of which factorisation: %.6f\n", s.t_factor_s);
      fprintf(out, " solve time without setup: %.6f\n", s.t_iterate_s);
      const dg_status ws = dg_write_solution(h, x.data());
      if (ws == DG_OK) fprintf(out, " solution written\n");
      if (prof) {
        FILE *pf = fopen(profname.c_str(), "w");
        if (pf) {
          fprintf(pf, "iterations %d\nsetup_host_s %.9f\nfactor_s %.9f\niterate_s %.9f\ntotal_s %.9f\n",
                  s.iterations, s.t_setup_s, s.t_factor_s, s.t_iterate_s, s.t_total_s);
          fprintf(pf, "subsolve_s %.9f\ncoarse_s %.9f\nspmv_s %.9f\ngpu_launches %d\n", s.t_subsolve_s,
                  s.t_coarse_s, s.t_spmv_s, s.gpu_launches);
          fclose(pf);
        }
      }
      rc = 0;
    }
  }
  dg_destroy(h);
  if (quiet) fclose(out);
  return rc;
}
