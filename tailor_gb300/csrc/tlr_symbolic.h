// tlr_symbolic.h -- nested-dissection ordering and multifrontal structure
// of the shift-and-invert matrix K = A_bc - sigma B_bc.
//
// The reference hands K to PETSc's PCLU / MUMPS (EigenSolver.cpp:61-71),
// whose orderings come from graph partitioners.  Here the graph is the
// structured (xi, eta) grid, so the separators are grid lines: a cut across
// xi is as wide as the symmetric xi coupling reach (5 lines in the
// interior of a q = 10 rule, up to 10 at the walls), a cut across the
// periodic eta ring is q_z / 2 lines wide and the ring needs one extra cut.
// Fronts are dense over whole grid nodes (5 unknowns each); a front's rows
// are its separator (pivot) nodes followed by its border: the nodes of
// ancestor separators adjacent to its box.
#pragma once

#include <cstdint>
#include <vector>

namespace tlr {

struct FrontInfo {
  int parent = -1;
  int height = 0;               // 0 for leaves
  std::vector<int> children;
  std::vector<int> piv;         // grid nodes eliminated here, in order
  std::vector<int> border;      // later-eliminated nodes, by elimination rank
  int p = 0, m = 0;             // scalar pivot count and front order
  long long off = 0;            // offset of the m x m front in the pool
  long long toff = 0;           // offset of the m-vector in the work pool
};

struct AsmEntry {               // one BSR block of K scattered into a front
  int k;                        // block index in A_bc's BSR values
  int row, col;                 // node positions inside the front
  int front;
  int bnode;                    // grid node whose B_bc block is subtracted, or -1
};

struct Symbolic {
  int ny = 0, nz = 0, nn = 0;
  std::vector<FrontInfo> fronts;        // postorder (children before parent)
  std::vector<int> rank;                // node -> elimination position
  std::vector<std::vector<int>> levels; // fronts by height
  std::vector<AsmEntry> entries;        // grouped by level, then front
  std::vector<long long> level_entry_begin;
  // extend-add: for front t, map of each child's border node -> position in t
  std::vector<int> cmap;                // concatenated maps
  std::vector<long long> cmap_off;      // per front (its map into the parent)
  long long pool_elems = 0;             // sum of m*m
  long long work_elems = 0;             // sum of m
  double flops = 0.0;                   // complex-counted (8 real per MAC)
  long long factor_elems = 0;           // sum p*(p + 2b)
};

// The solver's ring slack (percent).  Accepting a xi-cut of a ring box up
// to 1.1x the ring cut's nodes gives shallower top fronts: at 300 x 192 the
// factorisation needs 9% fewer flops (19.4 vs 21.3 TFLOP), the factor 2%
// fewer entries and the solves 12% fewer block steps than with the
// smallest separator (100), measured 8% faster to factorise.
constexpr int kRingSlackDefault = 110;

// Build the symbolic structure from the host copies of the rules and the
// BSR pattern (row_ptr / col of A_bc).  A box of the periodic ring is cut
// across xi instead of across the ring when the xi separator has at most
// ring_slack_percent / 100 times the ring cut's nodes.
int build_symbolic(int ny, int nz, const std::vector<int> &xi_idx, int sx,
                   const std::vector<int> &eta_off, int se,
                   const std::vector<int> &row_ptr, const std::vector<int> &col,
                   int leaf_nodes, Symbolic &out, int ring_slack_percent = kRingSlackDefault);

}  // namespace tlr
