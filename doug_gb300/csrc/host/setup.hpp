// Host-side setup of DOUG's two-level additive Schwarz preconditioner:
// control words, assembled input, strength of connection, aggregation,
// smoothed-aggregation restriction, Galerkin coarse matrix and overlapping
// subdomains.  This is the reference's np=1 semantics of doug_aggr
// (src/main/aggr.F90:124-215), restated on a CSR layout.  Everything here is
// integer / ordering work that the reference does sequentially on one rank;
// it runs once per matrix, before the GPU solve.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace dg {

// Shared + master control data (src/utils/globals.F90:85-154); -1 = unset.
struct Controls {
  int solver = -1, method = -1, fine_method = -1, num_iters = -1, coarse_method = -1;
  int num_subdomains = -1, levels = -1, overlap = -1, smoothers = -1, input_type = -1;
  int grid_size = -1, matrix_type = -1, initial_guess = -1, number_of_blocks = -1;
  int radius1 = -1, radius2 = -1, minasize1 = -1, minasize2 = -1, maxasize1 = -1, maxasize2 = -1;
  int debug = -1, verbose = -1, plotting = -1;
  double strong1 = -1.0, strong2 = -1.0, solve_tolerance = -1.0;
  int solve_maxiters = -1;
  bool symmstruct = false, symmnumeric = false;
  int interpolation_type = -1;
  int maxcie = -1, maxnd = -1, cutbal = -1, center_type = -1;  // geometric coarse grid (globals.F90:149-153)
  bool hanging_nodes = false;
  std::string assembled_mtx_file, assembled_rhs_file, solution_file;
  std::string info_file, elemmat_rhs_file, freedom_lists_file, coords_file, freemap_file;
  int assembled_mtx_format = -1, assembled_rhs_format = -1, solution_format = -1;
  int start_vec_type = -1;
  // extensions of this library (not reference control words)
  double omega = 0.33333333333333;  // prolongator smoother weight (CoarseMtx.F90:64)
  int precision = 0;                // 0 = FP64 path, 1 = mixed (FP32 factors)
  int replace_every = 50;           // residual replacement period (mixed path)
  int nd_leaf = 24;                 // nested-dissection leaf size of the subdomain factors
  int profile = 0;                  // 1: CUDA-event timing of the solve phases
  int reuse_factors = 0;            // 1: a solve after the first keeps the numeric factors
  int elemental_matvec = 0;         // 1: PCG products with the stored element matrices
  // tuning of the multifrontal batches (dg_autotune chooses them)
  int panel_rows = 512;             // fronts up to this size (and panel + E <= 96 KB): one CTA each
  int fwd_task_kb = 96;             // KB of E per forward task of a large front
  int lean_task_kb = 80;            // levels with smaller average tasks use 128-thread CTAs
  int thin_level_fronts = 1500;     // levels with fewer small fronts solve them one CTA per task
  int solve_schedule = 0;           // multifrontal solves: 0 one launch per level, 1 dependency-driven queue
  int solve_pdl = 1;                // 1: the level launches overlap through programmatic dependent launch
  int factor_overlap = 1;           // 1: a level's one-CTA fronts factored on a side stream beside its large fronts
  int executable = -1;              // which reference driver: -1/0 doug_aggr, 1 doug_geom
  int device_setup = 1;             // 1: smoothing, re-bucketing and Galerkin products on the GPU when one is visible
  int tensor_update = 1;            // FP32 super-panel trailing updates: 1 tcgen05 (TMEM accumulator), 0 mma.sync
  int super_panel = 128;           // columns of L per trailing update of a large front (multiple of 32)
  long long queue_wait_cycles = 1000000000LL;  // solve_schedule 1: limit of one dependency wait (cycles)
  int queue_skip_publish = -1;      // solve_schedule 1: forward entry whose done flag is withheld (failure tests)
};

// Parse one "name value" line the way util_actionOnCtrlArg does
// (DOUG_utils.F90:703-1150).  Returns false and fills err on a malformed value.
bool ctl_apply(Controls &c, const std::string &name, const std::string &value, std::string &err);
bool ctl_parse_text(Controls &c, const std::string &text, std::string &err);
// solve_maxiters default (DOUG_utils.F90:676-678); doug_geom always applies
// exact subdomain solves (geom.F90:101-102), whatever fine_method says
void ctl_finish(Controls &c);
bool parse_i10(const std::string &s, int &out);
bool parse_f10_5(const std::string &s, double &out);
bool parse_l1(const std::string &s, bool &out);

// Assembled input / vector / solution formats (SpMtx_class.F90:410-617,
// Vect.F90:840-947, DOUG_utils.F90:1598-1700).
bool read_assembled(const std::string &path, int format, int &n, std::vector<int> &ii,
                    std::vector<int> &jj, std::vector<double> &vv, std::string &err);
bool read_vector(const std::string &path, int format, int n, std::vector<double> &x,
                 std::string &err);
bool write_solution(const std::string &path, int format, const double *x, int n,
                    std::string &err);

// Structured input (input_type 3): the reference's generated test problem on
// one process (Distribution_struct.F90:36-147): the 5-point Laplacian
// (4 on the diagonal, -1 to the left, right, upper and lower neighbour that
// exist) on an n x n node grid, rows numbered row-major, entries of a row in
// the order diagonal, left, right, up, down; b = -1.  n < 1 means 100
// (Distribution.F90:69).
void structured_laplace(int n, int &nrows, std::vector<int> &ii, std::vector<int> &jj, std::vector<double> &vv,
                        std::vector<double> &b);

// Elemental input (input_type 1): element freedom lists and element matrices
// with right-hand sides.  Element e has the global freedoms (1-based)
// efree[eptr[e] .. eptr[e+1]) and the nfrelt x nfrelt matrix
// emat[emat_off[e] ..] stored column by column (the file's record j is
// column j), and the right-hand side erhs[eptr[e] ..].
struct ElementMesh {
  int nell = 0, ngf = 0, nsd = 0, mfrelt = 0, nnode = 0;
  std::vector<int> eptr, efree;
  std::vector<int64_t> emat_off;
  std::vector<double> emat, erhs;
};
// Reads info_file, freedom_lists_file and elemmat_rhs_file
// (Mesh.F90:293-460, ElemMtxs_distribute.F90:548-575): Fortran unformatted
// sequential records, little-endian.  number_of_blocks > 1 takes ngf from the
// largest freedom number, as the reference does.
bool read_elemental(const std::string &info, const std::string &freelists, const std::string &elemmat,
                    int number_of_blocks, ElementMesh &M, std::string &err);
bool check_elements(const ElementMesh &M, std::string &err);
// Assembles A and b the way one process does (ElemMtxs_assemble.F90:82-289):
// local freedoms are the freedoms used by some element in increasing global
// order; an entry exists where some element has a non-zero (i,j) and sums the
// elements' values in element order; b sums every element's right-hand side.
// The COO output walks the rows in order and each row's columns ascending,
// with the reference's flipped indices (row index = column freedom).  Indices
// are 1-based; lg_fmap[l] is the global freedom of local freedom l.
void assemble_elements(const ElementMesh &M, int &n, std::vector<int> &ii, std::vector<int> &jj,
                       std::vector<double> &vv, std::vector<double> &b, std::vector<int> &lg_fmap);

// Node coordinates for the geometric coarse grid (Mesh.F90:470-520):
// coordinate d of node v (1-based) at coords[(v-1)*nsd + d], and the node of
// global freedom f (1-based) at freemap[f-1].
struct NodeGeometry {
  int nsd = 0, nnode = 0;
  std::vector<double> coords;
  std::vector<int> freemap;
};
// coords_file: one record of nsd*nnode real64; freemap_file: one record of
// ngf int32 (Mesh_readFileCoords / Mesh_readFileFreemap)
bool read_geometry(const std::string &coords_path, const std::string &freemap_path, int nsd, int nnode, int ngf,
                   NodeGeometry &G, std::string &err);

// triplets in a definite order, 0-based
struct Coo {
  int nrows = 0, ncols = 0;
  std::vector<int> i, j;
  std::vector<double> v;
  size_t size() const { return v.size(); }
};

// CSR with DOUG's stable row arrangement (entries of a row keep their input order).
struct Csr {
  int nrows = 0, ncols = 0;
  std::vector<int64_t> ptr;
  std::vector<int> col;
  std::vector<double> val;
  int64_t nnz() const { return (int64_t)col.size(); }
};

struct Aggregates {
  int nagr = 0;
  std::vector<int> num;                 // 1-based aggregate per node, 0 = none
  std::vector<int> starts, nodes;       // 0-based CSR of nodes per aggregate (1-based ids)
};

struct SetupResult {
  int n = 0;
  Csr A;                                // fine matrix after the scale/unscale round trip
  std::vector<double> rhs;
  Aggregates fine, fine_full, coarse, coarse_full;
  Csr R;                                // restriction nagr x n, columns ascending per row
  Csr P;                                // prolongation n x nagr (= R^T), aggregates ascending
  Csr AC;                               // coarse matrix after its scale/unscale round trip
  std::vector<int64_t> sd_ptr;          // subdomain node lists (0-based offsets)
  std::vector<int> sd_nodes;            // 1-based node ids in DOUG order
  int overlap = 0, smoothers = 0, levels = 1;
  double strong1 = 0, strong2 = 0;
  int r1 = 0, r2 = 0, min1 = 0, max1 = 0, min2 = 0, max2 = 0;
  // R and AC in the reference's final COO order (for pattern export)
  std::vector<int> R_i, R_j, AC_i, AC_j;
  std::vector<double> R_v, AC_v;
  std::vector<double> coarse_xyz;       // geometric coarse grid: coordinates of R's coarse freedoms
  // setup phases (seconds): fine aggregation on the host (strength, aggregation),
  // restriction + Galerkin product (device time when they ran on the GPU)
  double t_aggregation = 0, t_coarse = 0;
  bool coarse_on_device = false;
};

// Robust coarse space (coarse_method 2): given A and the supports S_i of the
// coarse nodes (0-based node lists, support order), fill q (laid out as the
// supports) with q_i = A_i^-1 g(S_i), A_i = A(S_i, S_i), where g solves
// B g = 1 for B = sum_i R_i^T A_i^-1 R_i (RobustCoarseMtx.f90:53-210,
// pcg_robust.f90:37-120).  The product computes it on the GPU.
using RobustHook = std::function<bool(const Csr &A, const std::vector<int64_t> &supp_ptr,
                                      const std::vector<int> &supp_nodes, std::vector<double> &q,
                                      std::string &err)>;

// Build everything from 1-based COO triplets (assembled semantics: header
// swap and 0-based shift already applied by the caller).  part: optional
// 1-based partition vector (length n) that replaces the coarse-aggregate
// subdomains.  robust: the B-solve of coarse_method 2 (required for it).
// on_device: a GPU is visible, so with device_setup 1 (and coarse_method
// <= 1, smoothers <= 1) the restriction and Galerkin product run there.
// Returns false with err on a DOUG abort condition.
bool build_setup(const Controls &c_in, int n, const std::vector<int> &ii,
                 const std::vector<int> &jj, const std::vector<double> &vv,
                 const std::vector<int> *part, int nparts, SetupResult &out, std::string &err,
                 const RobustHook *robust = nullptr, bool on_device = false);

// doug_geom's setup on one process (geom.F90:62-116): subdomains = all
// unknowns (or the imported parts) with the overlap layers; levels 2 with
// elemental input (efree: the elements' global freedoms, lg_fmap: global
// freedom of every unknown, G: the node coordinates) adds the geometric
// coarse grid: R from geometric_restriction, AC = R A R^T.  R_i/R_j/R_v and
// AC_i/AC_j/AC_v hold them whole; the R, P and AC the solve uses keep only
// the coarse freedoms independent_coarse accepts.
bool build_setup_geom(const Controls &c, int n, const std::vector<int> &ii, const std::vector<int> &jj,
                      const std::vector<double> &vv, const std::vector<int> *part, int nparts,
                      const std::vector<int> *efree, const std::vector<int> *lg_fmap, const NodeGeometry *G,
                      SetupResult &out, std::string &err);
// The geometric coarse grid's restriction (coarse freedoms x unknowns,
// 0-based, the reference's entry order: unknown after unknown) and the
// coordinates of its coarse freedoms (nsd per freedom).
bool geometric_restriction(const Controls &c, const std::vector<int> &efree, const NodeGeometry &G,
                           const std::vector<int> &lg_fmap, Coo &R, std::vector<double> &coarse_xyz,
                           std::string &err);
// Coarse freedoms kept for the solve: a Cholesky of AC in natural order
// that skips pivots at or below 1e-10 of their diagonal (basis functions
// that depend on earlier ones); keep[i] = new 1-based number or 0.  More
// than 4000 coarse freedoms: all kept.
std::vector<int> independent_coarse(const Csr &AC);

// Smoothed aggregation over nodal blocks with a rigid-body near-nullspace
// (coarse_method 3, no reference counterpart): unode[u] is the 0-based mesh
// node of unknown u (its unknowns ascending are the node's components), xyz
// the node coordinates (nsd per node, indexed by that node id).  Needs an
// imported partition for the subdomains.
bool build_setup_rbm(const Controls &c, int n, const std::vector<int> &ii, const std::vector<int> &jj,
                     const std::vector<double> &vv, const std::vector<int> *part, int nparts,
                     const std::vector<int> &unode, int nsd, const std::vector<double> &xyz, SetupResult &out,
                     std::string &err);

// IntRestBuild with smoothers 0 or 1 (CoarseMtx.F90:50-233, 418-427) and
// CoarseMtxBuild (CoarseMtx.F90:476-516) on the GPU (dg_coarse_setup.cu):
// from the fine matrix A (row-arranged), its strong flags and the fine
// aggregates, fills out.R, out.P, out.R_i/R_j/R_v and AC with the same bits
// as the host path; seconds = the device time.  False with err on a CUDA
// error or when no device is visible.
bool device_restriction_galerkin(const Csr &A, const std::vector<char> &strong, const Aggregates &fine,
                                 int smoothers, double omega, SetupResult &out, Csr &AC, double &seconds,
                                 std::string &err);

// Batched independent systems: system k owns the rows [sys_row[k],
// sys_row[k+1]) and the triplets [sys_tri[k], sys_tri[k+1]) of (ii, jj, vv),
// whose indices are 1-based in the combined numbering.  Every system gets the
// setup of its own one-process run (build_setup on its own triplets; the
// systems run on parallel host threads); the result joins them as diagonal
// blocks: A, R, P and AC block-diagonal, aggregates and subdomains numbered
// after those of the systems before.
bool build_setup_systems(const Controls &c, const std::vector<int64_t> &sys_row,
                         const std::vector<int64_t> &sys_tri, const std::vector<int> &ii,
                         const std::vector<int> &jj, const std::vector<double> &vv, SetupResult &out,
                         std::string &err);

}  // namespace dg
