// Host-side structural setup of the SA-AMG hierarchy (see structure.h).
#include "structure.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>
#include <sstream>

namespace simp {

void finish_offsets(NodePattern& p, const std::vector<i32>& col_first) {
  p.off.resize(static_cast<size_t>(p.slots()));
  p.rowlen.assign(static_cast<size_t>(p.rows), 0);
#pragma omp parallel for schedule(static)
  for (i32 r = 0; r < p.rows; ++r) {
    i32 o = 0;
    for (i32 t = p.ptr[r]; t < p.ptr[r + 1]; ++t) {
      p.off[t] = o;
      o += col_first[p.nbr[t] + 1] - col_first[p.nbr[t]];
    }
    p.rowlen[r] = o;
  }
}

i64 scalar_nnz(const NodePattern& p, const std::vector<i32>& row_first) {
  i64 total = 0;
  for (i32 r = 0; r < p.rows; ++r)
    total += static_cast<i64>(row_first[r + 1] - row_first[r]) * p.rowlen[r];
  return total;
}

std::vector<i32> scalar_rowptr(const NodePattern& p, const std::vector<i32>& row_first) {
  const i32 n = row_first.back();
  std::vector<i32> ptr(static_cast<size_t>(n) + 1, 0);
  i64 acc = 0;
  for (i32 r = 0; r < p.rows; ++r)
    for (i32 i = row_first[r]; i < row_first[r + 1]; ++i) {
      acc += p.rowlen[r];
      if (acc > std::numeric_limits<i32>::max())
        throw Error(kBadInput, "matrix has more than 2^31-1 stored entries");
      ptr[i + 1] = static_cast<i32>(acc);
    }
  return ptr;
}

std::vector<i32> node_of_unknowns(const std::vector<i32>& first) {
  std::vector<i32> out(static_cast<size_t>(first.back()));
  for (size_t nd = 0; nd + 1 < first.size(); ++nd)
    for (i32 i = first[nd]; i < first[nd + 1]; ++i) out[i] = static_cast<i32>(nd);
  return out;
}

bool derive_node_pattern(i32 n, const i32* rowptr, const i32* col, const std::vector<i32>& first,
                         NodePattern& out, std::string& why) {
  const i32 nn = static_cast<i32>(first.size()) - 1;
  const std::vector<i32> node_of = node_of_unknowns(first);
  out = NodePattern();
  out.rows = out.cols = nn;
  out.ptr.assign(static_cast<size_t>(nn) + 1, 0);
  for (i32 I = 0; I < nn; ++I) {
    const i32 i0 = first[I];
    // columns of the node's first row, grouped by node
    i32 k = rowptr[i0];
    const i32 ke = rowptr[i0 + 1];
    i32 prev = -1;
    while (k < ke) {
      const i32 c = col[k];
      if (c < 0 || c >= n) { why = "column index out of range"; return false; }
      const i32 J = node_of[c];
      if (J <= prev) { why = "columns are not sorted by node"; return false; }
      const i32 sz = first[J + 1] - first[J];
      if (c != first[J] || ke - k < sz) { why = "a row does not cover whole column nodes"; return false; }
      for (i32 q = 0; q < sz; ++q)
        if (col[k + q] != first[J] + q) { why = "a row does not cover whole column nodes"; return false; }
      out.nbr.push_back(J);
      prev = J;
      k += sz;
    }
    out.ptr[I + 1] = static_cast<i32>(out.nbr.size());
    // the other rows of the node must repeat the same columns
    const i32 len = ke - rowptr[i0];
    for (i32 i = i0 + 1; i < first[I + 1]; ++i) {
      if (rowptr[i + 1] - rowptr[i] != len ||
          !std::equal(col + rowptr[i], col + rowptr[i + 1], col + rowptr[i0])) {
        std::ostringstream os;
        os << "the rows of node " << I << " do not share one column pattern";
        why = os.str();
        return false;
      }
    }
  }
  finish_offsets(out, first);
  return true;
}

i32 aggregate_nodes(const NodePattern& a, const std::vector<double>& acc,
                    const std::vector<double>& bdiag, double theta, std::vector<i32>& agg) {
  const i32 nn = a.rows;
  // Strong neighbours (other nodes only), ascending, with their strength.
  std::vector<i32> sptr(static_cast<size_t>(nn) + 1, 0), strong;
  std::vector<double> sval;
  strong.reserve(static_cast<size_t>(a.slots()));
  sval.reserve(static_cast<size_t>(a.slots()));
  for (i32 I = 0; I < nn; ++I) {
    const double di = bdiag[I];
    for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) {
      const i32 J = a.nbr[t];
      if (J == I) continue;
      const double s = std::sqrt(acc[t]);
      const double ref = std::sqrt(di * bdiag[J]);
      if (s > 0.0 && s >= theta * ref) {
        strong.push_back(J);
        sval.push_back(ref > 0.0 ? s / ref : 0.0);
      }
    }
    sptr[I + 1] = static_cast<i32>(strong.size());
  }
  agg.assign(static_cast<size_t>(nn), -1);
  i32 count = 0;
  // pass 1: a node whose strong neighbourhood is untouched seeds an aggregate
  for (i32 I = 0; I < nn; ++I) {
    if (agg[I] >= 0) continue;
    const i32 b = sptr[I], e = sptr[I + 1];
    if (b == e) continue;
    bool untouched = true;
    for (i32 k = b; k < e && untouched; ++k) untouched = agg[strong[k]] < 0;
    if (!untouched) continue;
    agg[I] = count;
    for (i32 k = b; k < e; ++k) agg[strong[k]] = count;
    ++count;
  }
  // pass 2: join the first-pass aggregate of the strongest such neighbour
  const std::vector<i32> first = agg;
  for (i32 I = 0; I < nn; ++I) {
    if (first[I] >= 0) continue;
    i32 best = -1;
    double bv = -1.0;
    for (i32 k = sptr[I]; k < sptr[I + 1]; ++k) {
      const i32 target = first[strong[k]];
      if (target >= 0 && sval[k] > bv) { best = target; bv = sval[k]; }
    }
    if (best >= 0) agg[I] = best;
  }
  // pass 3: what is left forms new aggregates with its unassigned neighbours
  for (i32 I = 0; I < nn; ++I) {
    if (agg[I] >= 0) continue;
    agg[I] = count;
    for (i32 k = sptr[I]; k < sptr[I + 1]; ++k)
      if (agg[strong[k]] < 0) agg[strong[k]] = count;
    ++count;
  }
  return count;
}

std::vector<double> rigid_body_modes(int dim, int ndpn, const std::vector<double>& coords,
                                     i32 num_nodes, const std::vector<i32>& unknowns) {
  const int m = dim == 2 ? 3 : 6;
  const i32 n = static_cast<i32>(unknowns.size());
  double lo[3] = {std::numeric_limits<double>::max(), std::numeric_limits<double>::max(),
                  std::numeric_limits<double>::max()};
  double hi[3] = {-lo[0], -lo[0], -lo[0]};
  for (i32 c = 0; c < num_nodes; ++c)
    for (int d = 0; d < 3; ++d) {
      const double x = d < dim ? coords[static_cast<size_t>(c) * dim + d] : 0.0;
      lo[d] = std::min(lo[d], x);
      hi[d] = std::max(hi[d], x);
    }
  double centre[3], scale = 0.0;
  for (int d = 0; d < 3; ++d) {
    centre[d] = 0.5 * (lo[d] + hi[d]);
    scale = std::max(scale, hi[d] - lo[d]);
  }
  scale = std::max(scale, 1.0e-300);
  std::vector<double> b(static_cast<size_t>(n) * m, 0.0);
  for (i32 i = 0; i < n; ++i) {
    const i32 g = unknowns[i];
    const i32 node = g / ndpn;
    const int k = g % ndpn;
    double r[3];
    for (int d = 0; d < 3; ++d) {
      const double x = d < dim ? coords[static_cast<size_t>(node) * dim + d] : 0.0;
      r[d] = (x - centre[d]) / scale;
    }
    double* row = &b[static_cast<size_t>(i) * m];
    row[k] = 1.0;
    if (dim == 2) {
      row[2] = k == 0 ? -r[1] : r[0];
    } else {
      // rotations about x, y, z: u = e_axis x r
      const double rx[3] = {0.0, -r[2], r[1]};
      const double ry[3] = {r[2], 0.0, -r[0]};
      const double rz[3] = {-r[1], r[0], 0.0};
      row[3] = rx[k];
      row[4] = ry[k];
      row[5] = rz[k];
    }
  }
  return b;
}

namespace {

// Householder QR with column pivoting (Businger-Golub, norm downdating of
// LAPACK xGEQPF / LAWN 176) of a column-major rows x m block; returns Q's
// first `rank` columns (column-major) and R P^T (rank x m, row-major).
void qr_block(std::vector<double>& a, i32 rows, int m, std::vector<double>& q,
              std::vector<double>& rp, i32& rank) {
  auto A = [&](i32 i, i32 j) -> double& { return a[static_cast<size_t>(j) * rows + i]; };
  const i32 size = std::min<i32>(rows, m);
  std::vector<double> tau(static_cast<size_t>(size), 0.0);
  std::vector<i32> perm(static_cast<size_t>(m));
  std::iota(perm.begin(), perm.end(), 0);
  std::vector<double> nu(static_cast<size_t>(m)), nd(static_cast<size_t>(m));
  for (i32 j = 0; j < m; ++j) {
    double s = 0.0;
    for (i32 i = 0; i < rows; ++i) s += A(i, j) * A(i, j);
    nu[j] = nd[j] = std::sqrt(s);
  }
  const double thresh = std::sqrt(std::numeric_limits<double>::epsilon());
  for (i32 k = 0; k < size; ++k) {
    i32 best = k;
    for (i32 j = k + 1; j < m; ++j) if (nu[j] > nu[best]) best = j;
    if (best != k) {
      for (i32 i = 0; i < rows; ++i) std::swap(A(i, k), A(i, best));
      std::swap(nu[k], nu[best]);
      std::swap(nd[k], nd[best]);
      std::swap(perm[k], perm[best]);
    }
    const double c0 = A(k, k);
    double tail = 0.0;
    for (i32 i = k + 1; i < rows; ++i) tail += A(i, k) * A(i, k);
    double beta, t;
    if (tail <= std::numeric_limits<double>::min()) {
      t = 0.0;
      beta = c0;
      for (i32 i = k + 1; i < rows; ++i) A(i, k) = 0.0;
    } else {
      beta = std::sqrt(c0 * c0 + tail);
      if (c0 >= 0.0) beta = -beta;
      const double inv = 1.0 / (c0 - beta);
      for (i32 i = k + 1; i < rows; ++i) A(i, k) *= inv;
      t = (beta - c0) / beta;
    }
    tau[k] = t;
    A(k, k) = beta;
    if (t != 0.0) {
      for (i32 j = k + 1; j < m; ++j) {
        double w = A(k, j);
        for (i32 i = k + 1; i < rows; ++i) w += A(i, k) * A(i, j);
        A(k, j) -= t * w;
        for (i32 i = k + 1; i < rows; ++i) A(i, j) -= t * A(i, k) * w;
      }
    }
    for (i32 j = k + 1; j < m; ++j) {
      if (nu[j] == 0.0) continue;
      double r = std::abs(A(k, j)) / nu[j];
      r = (1.0 + r) * (1.0 - r);
      if (r < 0.0) r = 0.0;
      const double ratio = nu[j] / nd[j];
      if (r * ratio * ratio <= thresh) {
        double s = 0.0;
        for (i32 i = k + 1; i < rows; ++i) s += A(i, j) * A(i, j);
        nd[j] = std::sqrt(s);
        nu[j] = nd[j];
      } else {
        nu[j] *= std::sqrt(r);
      }
    }
  }
  const double lead = size > 0 ? std::abs(A(0, 0)) : 0.0;
  rank = 0;
  for (i32 i = 0; i < size; ++i) if (std::abs(A(i, i)) > 1.0e-10 * lead) ++rank;
  rank = std::max<i32>(rank, 1);
  q.assign(static_cast<size_t>(rows) * rank, 0.0);
  auto Q = [&](i32 i, i32 j) -> double& { return q[static_cast<size_t>(j) * rows + i]; };
  for (i32 j = 0; j < rank; ++j) Q(j, j) = 1.0;
  for (i32 k = size - 1; k >= 0; --k) {
    if (tau[k] == 0.0) continue;
    for (i32 j = 0; j < rank; ++j) {
      double w = Q(k, j);
      for (i32 i = k + 1; i < rows; ++i) w += A(i, k) * Q(i, j);
      Q(k, j) -= tau[k] * w;
      for (i32 i = k + 1; i < rows; ++i) Q(i, j) -= tau[k] * A(i, k) * w;
    }
  }
  rp.assign(static_cast<size_t>(rank) * m, 0.0);
  for (i32 i = 0; i < rank; ++i)
    for (i32 k = 0; k < m; ++k)
      rp[static_cast<size_t>(i) * m + perm[k]] = (k >= i && i < rows) ? A(i, k) : 0.0;
}

}  // namespace

Tentative tentative_prolongator(const std::vector<i32>& first, const std::vector<i32>& agg,
                                i32 na, const std::vector<double>& null, int m) {
  const i32 nn = static_cast<i32>(first.size()) - 1;
  const i32 n = first.back();
  std::vector<i32> aptr(static_cast<size_t>(na) + 1, 0);
  for (i32 I = 0; I < nn; ++I) ++aptr[agg[I] + 1];
  for (i32 g = 0; g < na; ++g) aptr[g + 1] += aptr[g];
  std::vector<i32> anodes(static_cast<size_t>(nn));
  {
    std::vector<i32> fill(aptr.begin(), aptr.end() - 1);
    for (i32 I = 0; I < nn; ++I) anodes[fill[agg[I]]++] = I;
  }
  std::vector<std::vector<double>> qs(static_cast<size_t>(na)), rs(static_cast<size_t>(na));
  std::vector<i32> ranks(static_cast<size_t>(na), 0), rowsof(static_cast<size_t>(na), 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (i32 g = 0; g < na; ++g) {
    i32 rows = 0;
    for (i32 k = aptr[g]; k < aptr[g + 1]; ++k) rows += first[anodes[k] + 1] - first[anodes[k]];
    std::vector<double> block(static_cast<size_t>(rows) * m);
    i32 row = 0;
    for (i32 k = aptr[g]; k < aptr[g + 1]; ++k)
      for (i32 i = first[anodes[k]]; i < first[anodes[k] + 1]; ++i, ++row)
        for (int j = 0; j < m; ++j) block[static_cast<size_t>(j) * rows + row] = null[static_cast<size_t>(i) * m + j];
    qr_block(block, rows, m, qs[g], rs[g], ranks[g]);
    rowsof[g] = rows;
  }
  Tentative t;
  t.next_first.assign(static_cast<size_t>(na) + 1, 0);
  for (i32 g = 0; g < na; ++g) t.next_first[g + 1] = t.next_first[g] + ranks[g];
  const i32 nc = t.next_first.back();
  t.next_null.assign(static_cast<size_t>(nc) * m, 0.0);
  for (i32 g = 0; g < na; ++g)
    std::copy(rs[g].begin(), rs[g].end(), t.next_null.begin() + static_cast<long>(t.next_first[g]) * m);
  // per fine unknown: aggregate and local row
  t.phat_ptr.assign(static_cast<size_t>(n) + 1, 0);
  std::vector<i32> agg_of(static_cast<size_t>(n)), local(static_cast<size_t>(n));
  for (i32 g = 0; g < na; ++g) {
    i32 loc = 0;
    for (i32 k = aptr[g]; k < aptr[g + 1]; ++k)
      for (i32 i = first[anodes[k]]; i < first[anodes[k] + 1]; ++i) {
        agg_of[i] = g;
        local[i] = loc++;
      }
  }
  for (i32 i = 0; i < n; ++i) t.phat_ptr[i + 1] = t.phat_ptr[i] + ranks[agg_of[i]];
  t.phat.resize(static_cast<size_t>(t.phat_ptr.back()));
  for (i32 i = 0; i < n; ++i) {
    const i32 g = agg_of[i];
    for (i32 j = 0; j < ranks[g]; ++j)
      t.phat[static_cast<size_t>(t.phat_ptr[i]) + j] = qs[g][static_cast<size_t>(j) * rowsof[g] + local[i]];
  }
  return t;
}

NodePattern pattern_prolongator(const NodePattern& a, const std::vector<i32>& agg, i32 na) {
  NodePattern p;
  p.rows = a.rows;
  p.cols = na;
  p.ptr.assign(static_cast<size_t>(a.rows) + 1, 0);
  std::vector<std::vector<i32>> rows(static_cast<size_t>(a.rows));
#pragma omp parallel for schedule(static)
  for (i32 I = 0; I < a.rows; ++I) {
    std::vector<i32>& r = rows[I];
    for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) r.push_back(agg[a.nbr[t]]);
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
  }
  for (i32 I = 0; I < a.rows; ++I) p.ptr[I + 1] = p.ptr[I] + static_cast<i32>(rows[I].size());
  p.nbr.resize(static_cast<size_t>(p.ptr.back()));
#pragma omp parallel for schedule(static)
  for (i32 I = 0; I < a.rows; ++I) std::copy(rows[I].begin(), rows[I].end(), p.nbr.begin() + p.ptr[I]);
  return p;
}

NodePattern pattern_transpose(const NodePattern& p, std::vector<i32>* back) {
  NodePattern t;
  t.rows = p.cols;
  t.cols = p.rows;
  t.ptr.assign(static_cast<size_t>(p.cols) + 1, 0);
  for (i64 s = 0; s < p.slots(); ++s) ++t.ptr[p.nbr[s] + 1];
  for (i32 c = 0; c < p.cols; ++c) t.ptr[c + 1] += t.ptr[c];
  t.nbr.resize(static_cast<size_t>(p.slots()));
  if (back) back->resize(static_cast<size_t>(p.slots()));
  std::vector<i32> fill(t.ptr.begin(), t.ptr.end() - 1);
  for (i32 I = 0; I < p.rows; ++I)
    for (i32 s = p.ptr[I]; s < p.ptr[I + 1]; ++s) {
      const i32 q = fill[p.nbr[s]]++;
      t.nbr[q] = I;
      if (back) (*back)[q] = s;
    }
  return t;
}

NodePattern pattern_product(const NodePattern& a, const NodePattern& b) {
  NodePattern c;
  c.rows = a.rows;
  c.cols = b.cols;
  c.ptr.assign(static_cast<size_t>(a.rows) + 1, 0);
  std::vector<std::vector<i32>> rows(static_cast<size_t>(a.rows));
#pragma omp parallel
  {
    std::vector<i32> mark(static_cast<size_t>(b.cols), -1);
#pragma omp for schedule(dynamic, 1024)
    for (i32 I = 0; I < a.rows; ++I) {
      std::vector<i32>& r = rows[I];
      for (i32 t = a.ptr[I]; t < a.ptr[I + 1]; ++t) {
        const i32 J = a.nbr[t];
        for (i32 u = b.ptr[J]; u < b.ptr[J + 1]; ++u) {
          const i32 g = b.nbr[u];
          if (mark[g] != I) { mark[g] = I; r.push_back(g); }
        }
      }
      std::sort(r.begin(), r.end());
    }
  }
  for (i32 I = 0; I < a.rows; ++I) c.ptr[I + 1] = c.ptr[I] + static_cast<i32>(rows[I].size());
  c.nbr.resize(static_cast<size_t>(c.ptr.back()));
#pragma omp parallel for schedule(static)
  for (i32 I = 0; I < a.rows; ++I) {
    std::copy(rows[I].begin(), rows[I].end(), c.nbr.begin() + c.ptr[I]);
    std::vector<i32>().swap(rows[I]);
  }
  return c;
}

std::vector<i32> pattern_transpose_slots(const NodePattern& s) {
  std::vector<i32> tr(static_cast<size_t>(s.slots()), -1);
#pragma omp parallel for schedule(static)
  for (i32 I = 0; I < s.rows; ++I)
    for (i32 t = s.ptr[I]; t < s.ptr[I + 1]; ++t) {
      const i32 J = s.nbr[t];
      const i32* b = s.nbr.data() + s.ptr[J];
      const i32* e = s.nbr.data() + s.ptr[J + 1];
      const i32* hit = std::lower_bound(b, e, I);
      if (hit != e && *hit == I) tr[t] = static_cast<i32>(hit - s.nbr.data());
    }
  for (i32 v : tr)
    if (v < 0) throw Error(kBadInput, "multigrid: internal error, a Galerkin pattern is not symmetric");
  return tr;
}

std::vector<i32> pattern_self_slots(const NodePattern& s) {
  std::vector<i32> self(static_cast<size_t>(s.rows), -1);
  for (i32 I = 0; I < s.rows; ++I) {
    const i32* b = s.nbr.data() + s.ptr[I];
    const i32* e = s.nbr.data() + s.ptr[I + 1];
    const i32* hit = std::lower_bound(b, e, I);
    if (hit != e && *hit == I) self[I] = static_cast<i32>(hit - s.nbr.data());
  }
  return self;
}

double tridiagonal_max_eigenvalue(const std::vector<double>& a, const std::vector<double>& b) {
  const size_t k = a.size();
  if (k == 1) return a[0];
  double lo = std::numeric_limits<double>::max(), hi = -lo;
  for (size_t i = 0; i < k; ++i) {
    double r = 0.0;
    if (i > 0) r += std::abs(b[i - 1]);
    if (i + 1 < k) r += std::abs(b[i]);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  auto below = [&](double x) {
    size_t cnt = 0;
    double d = 1.0;
    for (size_t i = 0; i < k; ++i) {
      d = (a[i] - x) - (i > 0 ? b[i - 1] * b[i - 1] / d : 0.0);
      if (d == 0.0) d = -1e-300;
      if (d < 0.0) ++cnt;
    }
    return cnt;
  };
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (below(mid) == k) hi = mid; else lo = mid;
  }
  return 0.5 * (lo + hi);
}

}  // namespace simp
