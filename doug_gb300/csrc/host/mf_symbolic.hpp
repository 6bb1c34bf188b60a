// Symbolic analysis for the batched multifrontal Cholesky that replaces the
// reference's per-subdomain UMFPACK LU (src/solvers/Fact.F90:64-219,
// src/solvers/umfpack4wrap.c:196-256) and its coarse-matrix solve
// (src/solvers/subsolvers.F90:165-286).
//
// A "batch" is a set of independent sparse SPD matrices whose values come
// from one device array (the fine matrix values for the Schwarz subdomains,
// the coarse matrix values for the coarse solve).  Each matrix is ordered by
// nested dissection; every separator (and every leaf) is one dense front.
// Fronts of all matrices are grouped into levels of the assembly tree so that
// one kernel launch per level factors or solves every front of that level.
#pragma once
#include <cstdint>
#include <vector>

#include "setup.hpp"

namespace dg {

struct MfBatch {
  // per matrix
  int nmat = 0;
  std::vector<int64_t> xoff;      // offset of matrix m in the local-vector arena (nmat+1)
  // per local-vector position (new numbering, arena-wide)
  std::vector<int> gidx;          // 0-based global row (fine node / coarse node)
  // per front
  int nfronts = 0;
  std::vector<int64_t> f_off;     // dense m x m column-major front in the arena
  std::vector<int> f_m, f_k;
  std::vector<int64_t> f_rows;    // offset into rows (length m): local new-numbered rows
  std::vector<int64_t> f_xoff;    // xoff of the front's matrix
  std::vector<int> f_p0;          // first pivot (local new numbering)
  std::vector<int64_t> f_uoff;    // update vector offset (length m-k)
  std::vector<int64_t> f_woff;    // forward/backward work vector offset (length m)
  std::vector<int> f_child_ptr;   // children CSR (nfronts+1)
  std::vector<int> f_children;
  std::vector<int64_t> f_relmap;  // offset of this front's relmap (length m-k) into relmap
  std::vector<int64_t> f_asm;     // assembly entry range (nfronts+1)
  std::vector<int> f_parent;
  std::vector<int> f_level;
  std::vector<int> rows;          // all row lists
  std::vector<int> relmap;        // all relmaps
  std::vector<int64_t> asm_tgt;   // target offset in the front arena
  std::vector<int64_t> asm_sp;    // source range (entries+1)
  std::vector<int64_t> asm_src;   // value indices in the batch's value array
  // levels
  int nlevels = 0;
  std::vector<int> lvl_ptr;       // nlevels+1
  std::vector<int> lvl_fronts;    // fronts grouped by level
  std::vector<int> lvl_max_m;     // largest front per level
  int64_t arena = 0;              // front arena elements
  int64_t xlen = 0, ulen = 0, wlen = 0;
  int64_t factor_nnz = 0;         // stored factor entries (sum m*k - k(k-1)/2)
  double factor_flops = 0;        // partial Cholesky flops
  int max_m = 0;
};

struct MfOptions {
  int leaf = 64;                  // nested-dissection leaf size
};

// Subdomain batch: the principal submatrices A(inds, inds) of the fine matrix
// (DOUG's Factorise_subdomain, subsolvers.F90:104-163).  Value sources are
// positions in A.val.
void mf_build_subdomains(const Csr &A, const std::vector<int64_t> &sd_ptr,
                         const std::vector<int> &sd_nodes, const MfOptions &opt, MfBatch &out);

// Single-matrix batch for the coarse matrix (values from AC.val).
void mf_build_single(const Csr &M, const MfOptions &opt, MfBatch &out);

}  // namespace dg
