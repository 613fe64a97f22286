// Host-side, once-per-structure part of the SA-AMG setup: node-level
// sparsity patterns, strength-based aggregation, tentative prolongators and
// the symbolic Galerkin products.  Everything here is integer work (plus the
// small QR factorisations of the aggregates' near-null-space blocks); the
// numeric work of every setup runs on the GPU.
#pragma once

#include "common.h"

#include <string>
#include <vector>

namespace simp {

// Node-level pattern of a scalar CSR matrix whose rows of one node share a
// column list, grouped by whole column nodes (true of an assembled stiffness
// matrix and of every Galerkin product built from it).  Scalar row i of row
// node I holds, for each slot t in [ptr[I], ptr[I+1]), the columns
// col_first[nbr[t]] .. col_first[nbr[t] + 1] - 1 at offsets off[t] + k.
struct NodePattern {
  i32 rows = 0;              // row nodes
  i32 cols = 0;              // column nodes
  std::vector<i32> ptr;      // rows + 1
  std::vector<i32> nbr;      // column node of each slot, ascending per row
  std::vector<i32> off;      // offset of the slot's first column in the row
  std::vector<i32> rowlen;   // scalar row length, per row node
  i64 slots() const { return ptr.empty() ? 0 : ptr.back(); }
};

// off / rowlen from the column-node sizes.
void finish_offsets(NodePattern& p, const std::vector<i32>& col_first);
// Scalar rowptr (int32; throws when nnz exceeds the int32 range).
std::vector<i32> scalar_rowptr(const NodePattern& p, const std::vector<i32>& row_first);
i64 scalar_nnz(const NodePattern& p, const std::vector<i32>& row_first);

// Node-level pattern of a caller's CSR; false (with a reason) when the rows
// of a node do not share their columns or columns do not cover whole nodes.
bool derive_node_pattern(i32 n, const i32* rowptr, const i32* col, const std::vector<i32>& first,
                         NodePattern& out, std::string& why);

// Greedy three-pass aggregation of Vanek, Mandel and Brezina as the reference
// runs it (src/fem/Multigrid.cpp:457-565), from the block norms: acc[t] is
// the sum of squares of the slot's block (row node's rows, in order), bdiag
// the Frobenius norm of each node's diagonal block.  Returns the count.
i32 aggregate_nodes(const NodePattern& a, const std::vector<double>& acc,
                    const std::vector<double>& bdiag, double theta, std::vector<i32>& agg);

// Rigid-body near-null space of the finest level (Multigrid.cpp:383-455):
// n x m row-major, m = 3 (2-D) or 6 (3-D).
std::vector<double> rigid_body_modes(int dim, int ndpn, const std::vector<double>& coords,
                                     i32 num_nodes, const std::vector<i32>& unknowns);

// Tentative prolongator (Multigrid.cpp:567-669): per aggregate a pivoted
// Householder QR of its near-null-space rows.
struct Tentative {
  std::vector<i32> next_first;  // coarse unknowns of each aggregate (node_ptr)
  std::vector<i32> phat_ptr;    // per fine unknown: start of its rank values
  std::vector<double> phat;     // Q_a(local row, 0..rank)
  std::vector<double> next_null;  // coarse near-null space, nc x m row-major
};
Tentative tentative_prolongator(const std::vector<i32>& first, const std::vector<i32>& agg,
                                i32 num_aggs, const std::vector<double>& null, int m);

// Symbolic products at node level.
NodePattern pattern_prolongator(const NodePattern& a, const std::vector<i32>& agg, i32 num_aggs);
NodePattern pattern_transpose(const NodePattern& p, std::vector<i32>* back = nullptr);
NodePattern pattern_product(const NodePattern& a, const NodePattern& b);
// For a structurally symmetric square pattern: index of the (J, I) slot of
// every (I, J) slot.
std::vector<i32> pattern_transpose_slots(const NodePattern& s);
// Slot of the diagonal of every row node.
std::vector<i32> pattern_self_slots(const NodePattern& s);
// node_of[i] for every scalar unknown.
std::vector<i32> node_of_unknowns(const std::vector<i32>& first);

// Largest eigenvalue of a symmetric tridiagonal matrix by Sturm bisection.
double tridiagonal_max_eigenvalue(const std::vector<double>& diag, const std::vector<double>& off);

}  // namespace simp
