// extern "C" entry points of libsimp_gb300.so (declared in include/simp_gpu.h).
#include "../../include/simp_gpu.h"

#include "amg.h"
#include "autotune.h"
#include "problem.h"
#include "surrogate_net.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <thread>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

using namespace simp;

namespace {
thread_local std::string g_create_error;

AmgOptions convert(const simp_solver_options* o) {
  AmgOptions a;
  if (!o) return a;
  a.theta = o->strength_threshold;
  a.max_levels = o->max_levels;
  a.coarse_size = o->coarse_size;
  a.degree = o->smoother_degree;
  a.cheb_ratio = o->chebyshev_ratio;
  a.damping = o->prolongator_damping;
  a.lanczos_steps = o->lanczos_steps;
  a.pivot_tol = o->coarse_pivot_tolerance;
  a.reuse = o->reuse_aggregates != 0;
  a.rtol = o->iterative_tolerance;
  a.maxit = o->max_iterations > 0 ? o->max_iterations : 1000;
  a.precision = o->precision;
  a.graphs = o->cuda_graphs != 0;
  a.mf_transfer = o->matrix_free_transfer != 0;
  a.matrix_free = o->matrix_free;
  a.tensor_cores = o->tensor_cores;
  return a;
}

// Option checks of AmgPreconditioner's constructor (src/fem/Multigrid.cpp:907-925).
void validate(const AmgOptions& o) {
  if (!(o.theta >= 0.0 && o.theta < 1.0)) throw Error(kBadInput, "multigrid strength_threshold must lie in [0, 1)");
  if (o.max_levels < 1) throw Error(kBadInput, "multigrid max_levels must be at least 1");
  if (o.coarse_size < 1) throw Error(kBadInput, "multigrid coarse_size must be positive");
  if (o.degree < 1) throw Error(kBadInput, "multigrid smoother_degree must be at least 1");
  if (!(o.cheb_ratio > 1.0)) throw Error(kBadInput, "multigrid chebyshev_ratio must exceed 1");
  if (!(o.damping > 0.0 && o.damping < 2.0)) throw Error(kBadInput, "multigrid prolongator_damping must lie in (0, 2)");
  if (o.lanczos_steps < 2) throw Error(kBadInput, "multigrid lanczos_steps must be at least 2");
  if (!(o.rtol > 0.0)) throw Error(kBadInput, "the iterative tolerance must be positive");
  if (o.precision != SIMP_PRECISION_FP64 && o.precision != SIMP_PRECISION_MIXED)
    throw Error(kBadInput, "unknown precision mode");
  if (o.matrix_free < 0 || o.matrix_free > 2) throw Error(kBadInput, "matrix_free must be 0, 1 or 2");
  if (o.tensor_cores < 0 || o.tensor_cores > 1) throw Error(kBadInput, "tensor_cores must be 0 or 1");
}

template <class F>
int guarded(std::string& err, F&& f) {
  try {
    f();
    return kOk;
  } catch (const Error& e) {
    err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    err = "out of host memory";
    return kBadInput;
  } catch (const std::exception& e) {
    err = e.what();
    return kBadInput;
  }
}

void use_device(int dev) { SIMP_CUDA(cudaSetDevice(dev)); }

// One history row (TopologyIteration) from an evaluation and an update.
void fill_record(const GpuProblem& g, const Evaluation& ev, const OcStep& st, double seconds,
                 simp_iteration_record* rec) {
  rec->compliance = ev.compliance;
  rec->volume_fraction = ev.volume_fraction;
  rec->max_change = st.max_change;
  rec->lambda = st.lambda;
  rec->gray_level = g.gray;
  rec->linear_iterations = ev.linear_iterations;
  rec->bisections = st.bisections;
  rec->seconds = seconds;
  // MMA: the volume row fval(0) <= constraint_tolerance (1e-4)
  const double fval0 = g.d.robust ? ev.volume_dilated / g.dilated_target - 1.0 : ev.volume_fraction / g.d.vf - 1.0;
  rec->volume_converged = g.d.optimizer == 1 ? (fval0 <= 1.0e-4 ? 1 : 0) : (st.converged ? 1 : 0);
  rec->final_stage = g.beta_at_final() ? 1 : 0;
  rec->beta = g.d.projection ? g.beta : 0.0;
  rec->eroded_volume_fraction = rec->dilated_volume_fraction = rec->dilated_target_fraction = 0.0;
  if (g.d.robust) {
    rec->volume_fraction = ev.volume_intermediate / g.domain_volume;
    rec->eroded_volume_fraction = ev.volume_fraction;
    rec->dilated_volume_fraction = ev.volume_dilated / g.domain_volume;
    rec->dilated_target_fraction = g.dilated_target / g.domain_volume;
  }
}

}  // namespace

struct simp_ctx {
  AmgOptions opt;
  int device = 0;
  std::unique_ptr<GpuAmg> amg;
  int dim = 0, ndpn = 0;
  std::vector<double> coords;
  i32 num_nodes = 0;
  std::vector<i32> unknowns;
  bool has_layout = false, layout_changed = true;
  i32 fp_n = -1;
  i64 fp_nnz = -1;
  std::string err;
  DBuf<double> db, dx;
  // simp_set_pattern / simp_set_values(_device) / simp_setup
  std::vector<i32> pat_rowptr, pat_col;
  std::vector<double> host_values;
  const double* device_values = nullptr;
};

struct simp_problem {
  std::unique_ptr<GpuProblem> p;
  int device = 0;
  std::string err;
  std::vector<std::string> modal_warnings, buckling_warnings;
};

extern "C" {

void simp_default_options(simp_solver_options* o) {
  o->strength_threshold = 0.02;
  o->max_levels = 12;
  o->coarse_size = 1500;
  o->smoother_degree = 3;
  o->chebyshev_ratio = 30.0;
  o->prolongator_damping = 4.0 / 3.0;
  o->lanczos_steps = 12;
  o->coarse_pivot_tolerance = 1.0e-13;
  o->reuse_aggregates = 1;
  o->iterative_tolerance = 1.0e-12;
  o->max_iterations = 0;
  o->precision = SIMP_PRECISION_FP64;
  o->device = 0;
  o->cuda_graphs = 1;
  o->matrix_free_transfer = 1;
  o->matrix_free = 1;
  o->tensor_cores = 0;
}

int simp_ctx_create(const simp_solver_options* opts, simp_ctx** out) {
  return guarded(g_create_error, [&] {
    if (!out) throw Error(kBadInput, "simp_ctx_create: out is NULL");
    std::unique_ptr<simp_ctx> c(new simp_ctx());
    simp_solver_options def;
    simp_default_options(&def);
    c->opt = convert(opts ? opts : &def);
    validate(c->opt);
    c->device = opts ? opts->device : 0;
    use_device(c->device);
    c->amg.reset(new GpuAmg(c->opt));
    *out = c.release();
  });
}

void simp_ctx_destroy(simp_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  delete ctx;
}

const char* simp_last_error(const simp_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int simp_set_layout(simp_ctx* ctx, int32_t dim, int32_t ndpn, const double* coords, int32_t num_nodes,
                    const int32_t* unknowns, int32_t n) {
  return guarded(ctx->err, [&] {
    if (dim != 2 && dim != 3) throw Error(kBadInput, "multigrid: the DOF layout must be two- or three-dimensional");
    const int nd = ndpn > 0 ? ndpn : dim;
    if (nd != dim) {
      std::ostringstream os;
      os << "multigrid: a " << dim << "-D layout with " << nd
         << " DOFs per node is not supported by the GPU solver (translations only)";
      throw Error(kBadInput, os.str());
    }
    if (!coords || !unknowns || num_nodes < 0 || n < 0) throw Error(kBadInput, "multigrid: incomplete DOF layout");
    std::vector<double> c(coords, coords + static_cast<size_t>(num_nodes) * dim);
    std::vector<i32> u(unknowns, unknowns + n);
    const bool same = ctx->has_layout && ctx->dim == dim && ctx->ndpn == nd && c == ctx->coords && u == ctx->unknowns;
    if (!same) {
      ctx->dim = dim;
      ctx->ndpn = nd;
      ctx->coords.swap(c);
      ctx->unknowns.swap(u);
      ctx->num_nodes = num_nodes;
      ctx->layout_changed = true;
    }
    ctx->has_layout = true;
  });
}

namespace {

// factorize with the values either on the host or on the device (exactly one
// of host_values / device_values is non-null)
void factorize_impl(simp_ctx* ctx, int32_t n, const int32_t* rowptr, const int32_t* colidx,
                    const double* host_values, const double* device_values) {
    const std::string who = "AMG-CG(chebyshev, GPU)";
    const double* values = host_values;
    std::vector<double> staged;
    if (n <= 0 || !rowptr) throw Error(kBadInput, who + " received an empty system");
    if (!ctx->has_layout)
      throw Error(kBadInput, who + " needs the DOF layout (node coordinates of the unknowns) to build its "
                                   "rigid-body near-null space; the caller did not supply one");
    if (static_cast<i32>(ctx->unknowns.size()) != n) {
      std::ostringstream os;
      os << "multigrid: the DOF layout lists " << ctx->unknowns.size() << " unknowns for a matrix of " << n << " rows";
      throw Error(kBadInput, os.str());
    }
    const i64 nnz = rowptr[n];
    if (rowptr[0] != 0 || nnz <= 0) throw Error(kBadInput, "multigrid: malformed row pointer");
    GpuAmg& amg = *ctx->amg;
    const bool same = amg.ready() && ctx->fp_n == n && ctx->fp_nnz == nnz && !ctx->layout_changed;
    if (!values && !same) {
      // device values: the host checks (finite, symmetric) of a new structure
      staged.resize(static_cast<size_t>(nnz));
      SIMP_CUDA(cudaMemcpy(staged.data(), device_values, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
      values = staged.data();
    }
    if (values)
      for (i64 k = 0; k < nnz; ++k)
        if (!std::isfinite(values[k]))
          throw Error(kNonFinite, "multigrid: the system matrix has a non-finite entry");
    if (!same) {
      // symmetry check once per structure (Multigrid.cpp:968-991)
      double mx = 0.0;
      for (i64 k = 0; k < nnz; ++k) mx = std::max(mx, std::abs(values[k]));
      for (i32 i = 0; i < n; ++i)
        for (i32 k = rowptr[i]; k < rowptr[i + 1]; ++k) {
          const i32 j = colidx[k];
          if (j < 0 || j >= n) throw Error(kBadInput, "multigrid: column index out of range");
          const i32* b = colidx + rowptr[j];
          const i32* e = colidx + rowptr[j + 1];
          const i32* hit = std::lower_bound(b, e, i);
          const double other = (hit != e && *hit == i) ? values[hit - colidx] : 0.0;
          if (std::abs(other - values[k]) > 1.0e-10 * mx) {
            std::ostringstream os;
            os << "multigrid: the system matrix is not symmetric (entry (" << i << ", " << j << ") = " << values[k]
               << " but (" << j << ", " << i << ") = " << other
               << "); conjugate gradients needs a symmetric positive-definite matrix";
            throw Error(kBadInput, os.str());
          }
        }
      // unknowns grouped by node (Multigrid.cpp:383-412)
      std::vector<i32> first(1, 0);
      i32 prev = -1;
      for (i32 i = 0; i < n; ++i) {
        const i32 g = ctx->unknowns[i];
        const i32 node = g / ctx->ndpn;
        if (g < 0 || node >= ctx->num_nodes) {
          std::ostringstream os;
          os << "multigrid: unknown " << i << " maps to DOF " << g << ", outside the model's " << ctx->num_nodes
             << " nodes";
          throw Error(kBadInput, os.str());
        }
        if (i > 0 && g <= ctx->unknowns[i - 1])
          throw Error(kBadInput, "multigrid: the DOF layout must list unknowns in ascending order");
        if (node != prev) {
          if (i > 0) first.push_back(i);
          prev = node;
        }
      }
      first.push_back(n);
      NodePattern pat;
      std::string why;
      if (!derive_node_pattern(n, rowptr, colidx, first, pat, why))
        throw Error(kBadInput, "multigrid: the matrix pattern is not node-blocked (" + why + ")");
      const std::vector<i32> self = pattern_self_slots(pat);
      for (size_t I = 0; I < self.size(); ++I)
        if (self[I] < 0) {
          std::ostringstream os;
          os << "multigrid: node " << I << " has no diagonal block; a stiffness matrix must have a "
                "positive diagonal";
          throw Error(kBreakdown, os.str());
        }
      amg.levels.clear();
      Level& l0 = amg.level0();
      l0.n = n;
      l0.nnodes = static_cast<i32>(first.size()) - 1;
      l0.first = first;
      l0.apat = std::move(pat);
      l0.d_first.upload(l0.first, amg.stream);
      l0.d_node_of.upload(node_of_unknowns(l0.first), amg.stream);
      l0.d_apat.upload(l0.apat, amg.stream);
      l0.d_self.upload(pattern_self_slots(l0.apat), amg.stream);
      l0.a.rows = l0.a.cols = n;
      l0.a.nnz = nnz;
      l0.a.ptr.upload(rowptr, static_cast<size_t>(n) + 1, amg.stream);
      l0.a.col.upload(colidx, static_cast<size_t>(nnz), amg.stream);
      l0.null = rigid_body_modes(ctx->dim, ctx->ndpn, ctx->coords, ctx->num_nodes, ctx->unknowns);
    }
    Level& l0 = *amg.levels.front();
    if (host_values) {
      l0.a.v64.upload(host_values, static_cast<size_t>(nnz), amg.stream);
    } else {
      l0.a.v64.alloc(static_cast<size_t>(nnz));
      SIMP_CUDA(cudaMemcpyAsync(l0.a.v64.p, device_values, sizeof(double) * nnz, cudaMemcpyDeviceToDevice,
                                amg.stream));
    }
    amg.setup(!same);
    ctx->fp_n = n;
    ctx->fp_nnz = nnz;
    ctx->layout_changed = false;
}

}  // namespace

int simp_factorize(simp_ctx* ctx, int32_t n, const int32_t* rowptr, const int32_t* colidx, const double* values) {
  return guarded(ctx->err, [&] {
    use_device(ctx->device);
    if (!values) throw Error(kBadInput, "AMG-CG(chebyshev, GPU) received no matrix values");
    factorize_impl(ctx, n, rowptr, colidx, values, nullptr);
  });
}

int simp_set_pattern(simp_ctx* ctx, int32_t n, const int32_t* rowptr, const int32_t* colidx) {
  return guarded(ctx->err, [&] {
    if (n <= 0 || !rowptr || !colidx) throw Error(kBadInput, "AMG-CG(chebyshev, GPU) received an empty pattern");
    if (rowptr[0] != 0 || rowptr[n] <= 0) throw Error(kBadInput, "multigrid: malformed row pointer");
    ctx->pat_rowptr.assign(rowptr, rowptr + n + 1);
    ctx->pat_col.assign(colidx, colidx + rowptr[n]);
    ctx->host_values.clear();
    ctx->device_values = nullptr;
  });
}

int simp_set_values(simp_ctx* ctx, const double* values) {
  return guarded(ctx->err, [&] {
    if (ctx->pat_rowptr.empty()) throw Error(kBadInput, "simp_set_values needs simp_set_pattern first");
    if (!values) throw Error(kBadInput, "simp_set_values received no values");
    ctx->host_values.assign(values, values + ctx->pat_col.size());
    ctx->device_values = nullptr;
  });
}

int simp_set_values_device(simp_ctx* ctx, const double* values_device) {
  return guarded(ctx->err, [&] {
    if (ctx->pat_rowptr.empty()) throw Error(kBadInput, "simp_set_values_device needs simp_set_pattern first");
    if (!values_device) throw Error(kBadInput, "simp_set_values_device received no values");
    ctx->host_values.clear();
    ctx->device_values = values_device;
  });
}

int simp_setup(simp_ctx* ctx) {
  return guarded(ctx->err, [&] {
    use_device(ctx->device);
    if (ctx->pat_rowptr.empty()) throw Error(kBadInput, "simp_setup needs simp_set_pattern first");
    if (ctx->host_values.empty() && !ctx->device_values)
      throw Error(kBadInput, "simp_setup needs simp_set_values or simp_set_values_device first");
    const i32 n = static_cast<i32>(ctx->pat_rowptr.size()) - 1;
    factorize_impl(ctx, n, ctx->pat_rowptr.data(), ctx->pat_col.data(),
                   ctx->host_values.empty() ? nullptr : ctx->host_values.data(), ctx->device_values);
  });
}

int simp_solve(simp_ctx* ctx, int32_t nrhs, const double* B, const double* X0, double* X, int32_t* iterations,
               double* relres) {
  return guarded(ctx->err, [&] {
    use_device(ctx->device);
    GpuAmg& amg = *ctx->amg;
    if (!amg.ready()) throw Error(kBadInput, "AMG-CG(chebyshev, GPU): solve called before factorize");
    const i32 n = amg.levels.front()->n;
    ctx->db.alloc(n);
    ctx->dx.alloc(n);
    for (int k = 0; k < nrhs; ++k) {
      ctx->db.upload(B + static_cast<size_t>(k) * n, n, amg.stream);
      if (X0) ctx->dx.upload(X0 + static_cast<size_t>(k) * n, n, amg.stream);
      else ctx->dx.zero(amg.stream);
      const GpuAmg::PcgResult r = amg.solve(ctx->db.p, ctx->dx.p);
      ctx->dx.download(X + static_cast<size_t>(k) * n, n, amg.stream);
      SIMP_CUDA(cudaStreamSynchronize(amg.stream));
      if (iterations) iterations[k] = r.iterations;
      if (relres) relres[k] = r.relres;
      if (!r.converged) {
        std::ostringstream os;
        os << "AMG-CG(chebyshev, GPU) did not converge: " << r.iterations
           << " iterations left a relative residual of " << r.relres << " against a tolerance of " << amg.opt.rtol
           << " (" << amg.levels.size() << " levels, operator complexity " << amg.stats.operator_complexity
           << "). Raise solver.linear.max_iterations, lower solver.linear.amg.strength_threshold, raise "
              "amg.smoother_degree, or use \"simplicial_ldlt\"";
        throw Error(kMaxIter, os.str());
      }
    }
  });
}

int simp_apply_preconditioner(simp_ctx* ctx, const double* r, double* z) {
  return guarded(ctx->err, [&] {
    use_device(ctx->device);
    GpuAmg& amg = *ctx->amg;
    if (!amg.ready()) throw Error(kBadInput, "multigrid: apply() called before setup()");
    const i32 n = amg.levels.front()->n;
    ctx->db.upload(r, n, amg.stream);
    ctx->dx.alloc(n);
    amg.apply(ctx->db.p, ctx->dx.p);
    ctx->dx.download(z, n, amg.stream);
    SIMP_CUDA(cudaStreamSynchronize(amg.stream));
  });
}

static void fill_stats(const GpuAmg& amg, simp_amg_stats* s) {
  std::memset(s, 0, sizeof(*s));
  s->num_levels = amg.stats.num_levels;
  s->reused_aggregates = amg.stats.reused ? 1 : 0;
  s->operator_complexity = amg.stats.operator_complexity;
  s->grid_complexity = amg.stats.grid_complexity;
  s->coarse_pivot_ratio = amg.stats.pivot_ratio;
  s->setup_seconds = amg.stats.setup_seconds;
  s->storage_nonzeros = amg.stats.storage;
  for (size_t k = 0; k < amg.levels.size() && k < 16; ++k) {
    s->level_rows[k] = amg.levels[k]->n;
    s->level_nnz[k] = amg.levels[k]->a.nnz;
    s->level_aggregates[k] = k + 1 < amg.levels.size() ? amg.levels[k + 1]->nnodes : 0;
    s->level_lambda[k] = amg.levels[k]->lambda;
  }
}

int simp_stats(simp_ctx* ctx, simp_amg_stats* s) {
  return guarded(ctx->err, [&] { fill_stats(*ctx->amg, s); });
}

static void copy_level_matrix(GpuAmg& amg, int level, int32_t* rows, int64_t* nnz, int32_t* rowptr, int32_t* col,
                              double* val) {
  if (level < 0 || level >= static_cast<int>(amg.levels.size())) throw Error(kBadInput, "no such level");
  const Level& lv = *amg.levels[level];
  if (rows) *rows = lv.n;
  if (nnz) *nnz = lv.a.nnz;
  if (rowptr) lv.a.ptr.download(rowptr, static_cast<size_t>(lv.n) + 1, amg.stream);
  if (col) lv.a.col.download(col, static_cast<size_t>(lv.a.nnz), amg.stream);
  if (val) lv.a.v64.download(val, static_cast<size_t>(lv.a.nnz), amg.stream);
  SIMP_CUDA(cudaStreamSynchronize(amg.stream));
}

int simp_level_aggregates(simp_ctx* ctx, int32_t level, int32_t* agg, int32_t* count) {
  return guarded(ctx->err, [&] {
    GpuAmg& amg = *ctx->amg;
    if (level < 0 || level >= static_cast<int>(amg.levels.size())) throw Error(kBadInput, "no such level");
    const Level& lv = *amg.levels[level];
    if (count) *count = lv.nnodes;
    if (agg) {
      if (lv.agg.empty()) std::fill(agg, agg + lv.nnodes, -1);
      else std::copy(lv.agg.begin(), lv.agg.end(), agg);
    }
  });
}

int simp_level_matrix(simp_ctx* ctx, int32_t level, int32_t* rows, int64_t* nnz, int32_t* rowptr, int32_t* col,
                      double* val) {
  return guarded(ctx->err, [&] {
    use_device(ctx->device);
    copy_level_matrix(*ctx->amg, level, rows, nnz, rowptr, col, val);
  });
}

int simp_level_prolongator(simp_ctx* ctx, int32_t level, int32_t* rows, int32_t* cols, int64_t* nnz,
                           int32_t* rowptr, int32_t* col, double* val) {
  return guarded(ctx->err, [&] {
    use_device(ctx->device);
    GpuAmg& amg = *ctx->amg;
    if (level < 0 || level + 1 >= static_cast<int>(amg.levels.size())) throw Error(kBadInput, "no such transfer level");
    const Level& lv = *amg.levels[level];
    if (rows) *rows = lv.p.rows;
    if (cols) *cols = lv.p.cols;
    if (nnz) *nnz = lv.p.nnz;
    if (rowptr) lv.p.ptr.download(rowptr, static_cast<size_t>(lv.p.rows) + 1, amg.stream);
    if (col) lv.p.col.download(col, static_cast<size_t>(lv.p.nnz), amg.stream);
    if (val) lv.p.v64.download(val, static_cast<size_t>(lv.p.nnz), amg.stream);
    SIMP_CUDA(cudaStreamSynchronize(amg.stream));
  });
}

// ---- whole SIMP iteration ----

int simp_problem_create(const simp_problem_desc* dsc, const simp_solver_options* opts, simp_problem** out) {
  return guarded(g_create_error, [&] {
    if (!dsc || !out) throw Error(kBadInput, "simp_problem_create: NULL argument");
    simp_solver_options def;
    simp_default_options(&def);
    const simp_solver_options* o = opts ? opts : &def;
    AmgOptions ao = convert(o);
    validate(ao);
    // the descriptor is checked on the host before the device is touched
    ProblemDesc d;
    d.dim = dsc->dim;
    d.nx = dsc->nx;
    d.ny = dsc->ny;
    d.nz = dsc->dim == 3 ? dsc->nz : 1;
    d.lx = dsc->lx;
    d.ly = dsc->ly;
    d.lz = dsc->lz;
    d.thickness = dsc->thickness;
    if (d.dim != 2 && d.dim != 3) throw Error(kBadInput, "dim must be 2 or 3");
    const int ed = d.dim == 3 ? 24 : 8;
    if (!dsc->element_matrix || !dsc->fixed || !dsc->loads || !dsc->weights)
      throw Error(kBadInput, "simp_problem_create: missing element matrix, supports or loads");
    d.ke.assign(dsc->element_matrix, dsc->element_matrix + ed * ed);
    const i64 nn = static_cast<i64>(d.nx + 1) * (d.ny + 1) * (d.dim == 3 ? d.nz + 1 : 1);
    const i64 ndof = nn * d.dim;
    d.fixed.assign(dsc->fixed, dsc->fixed + ndof);
    d.nloads = dsc->num_loads;
    if (d.nloads < 1) throw Error(kBadInput, "at least one load case is needed");
    d.loads.assign(dsc->loads, dsc->loads + ndof * d.nloads);
    double ws = 0.0;
    for (int l = 0; l < d.nloads; ++l) ws += dsc->weights[l];
    if (!(ws > 0.0)) throw Error(kBadInput, "load-case weights must have a positive sum");
    for (int l = 0; l < d.nloads; ++l) d.weights.push_back(dsc->weights[l] / ws);
    d.radius = dsc->filter_radius;
    d.vf = dsc->volume_fraction;
    if (!(d.vf > 0.0 && d.vf <= 1.0)) throw Error(kBadInput, "volume fraction must lie in (0, 1]");
    d.x0 = dsc->initial_density >= 0.0 ? dsc->initial_density : dsc->volume_fraction;
    d.penalty = dsc->penalty;
    // SimpOptions::validate (src/topopt/SimpInterpolation.cpp:31-44)
    if (!(d.penalty >= 1.0)) {
      std::ostringstream os;
      os << "SIMP penalty must be >= 1 (got " << d.penalty << ")";
      throw Error(kBadInput, os.str());
    }
    d.emin = dsc->emin_ratio;
    if (!(d.emin > 0.0 && d.emin < 1.0)) throw Error(kBadInput, "SIMP emin_ratio must lie in (0, 1)");
    d.move = dsc->move_limit;
    if (!(d.move > 0.0 && d.move <= 1.0)) throw Error(kBadInput, "optimizer.move_limit must lie in (0, 1]");
    d.damping = dsc->damping;
    if (!(d.damping > 0.0 && d.damping <= 1.0)) throw Error(kBadInput, "optimizer.damping must lie in (0, 1]");
    if (dsc->warm_start < 0 || dsc->warm_start > 3) throw Error(kBadInput, "warm_start must be 0, 1, 2 or 3");
    d.warm = dsc->warm_start;
    if (dsc->block_pcg < 0 || dsc->block_pcg > 2) throw Error(kBadInput, "block_pcg must be 0, 1 or 2");
    d.block_pcg = dsc->block_pcg;
    d.projection = dsc->projection != 0;
    if (d.projection) {
      // ProjectionOptions::validate (src/topopt/Projection.cpp:10-43)
      std::ostringstream os;
      if (!(dsc->eta > 0.0 && dsc->eta < 1.0)) os << "projection eta must lie in (0, 1), got " << dsc->eta;
      else if (!(dsc->beta_start > 0.0) || !std::isfinite(dsc->beta_start))
        os << "projection beta_start must be positive, got " << dsc->beta_start;
      else if (!(dsc->beta_max >= dsc->beta_start) || !std::isfinite(dsc->beta_max))
        os << "projection beta_max (" << dsc->beta_max << ") must be at least beta_start (" << dsc->beta_start
           << ")";
      else if (dsc->beta_max > 1024.0)
        os << "projection beta_max = " << dsc->beta_max << " is beyond any useful sharpness";
      else if (!(dsc->beta_factor > 1.0)) os << "projection beta_factor must exceed 1, got " << dsc->beta_factor;
      else if (dsc->beta_interval < 1)
        os << "projection beta_interval must be at least 1, got " << dsc->beta_interval;
      if (!os.str().empty()) throw Error(kBadInput, os.str());
      d.eta = dsc->eta;
      d.beta_start = dsc->beta_start;
      d.beta_max = dsc->beta_max;
      d.beta_factor = dsc->beta_factor;
      d.beta_interval = dsc->beta_interval;
      d.advance_on_convergence = dsc->advance_on_convergence != 0;
      d.change_tol = dsc->change_tolerance;
    }
    d.robust = dsc->robust != 0;
    if (d.robust) {
      if (!d.projection) throw Error(kBadInput, "projection.robust needs the projection enabled");
      if (!(dsc->eta - dsc->robust_delta > 0.0 && dsc->eta + dsc->robust_delta < 1.0 && dsc->robust_delta > 0.0))
        throw Error(kBadInput, "projection.robust_delta must keep eta - delta and eta + delta inside (0, 1)");
      if (dsc->robust_volume_interval < 1) throw Error(kBadInput, "projection.robust_volume_interval must be >= 1");
      d.robust_delta = dsc->robust_delta;
      d.robust_interval = dsc->robust_volume_interval;
    }
    if (dsc->optimizer != 0 && dsc->optimizer != 1) throw Error(kBadInput, "unknown optimizer (expected 0 OC, 1 MMA)");
    d.optimizer = dsc->optimizer;
    if (dsc->warm_history < 0 || dsc->warm_history > kHistory) throw Error(kBadInput, "warm_history must be 0 .. 3");
    d.warm_history = dsc->warm_history > 0 ? dsc->warm_history : kHistory;
    use_device(o->device);
    std::unique_ptr<simp_problem> p(new simp_problem());
    p->device = o->device;
    p->p.reset(new GpuProblem(d, ao));
    *out = p.release();
  });
}

void simp_problem_destroy(simp_problem* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  delete p;
}

const char* simp_problem_last_error(const simp_problem* p) { return p ? p->err.c_str() : g_create_error.c_str(); }

int simp_problem_sizes(simp_problem* p, int64_t* s) {
  return guarded(p->err, [&] {
    s[0] = p->p->ne;
    s[1] = p->p->nn;
    s[2] = p->p->ndof;
    s[3] = p->p->nfree;
    s[4] = p->p->amg.levels.front()->a.nnz;
  });
}

int simp_set_design(simp_problem* p, const double* x) {
  return guarded(p->err, [&] {
    use_device(p->device);
    for (i64 e = 0; e < p->p->ne; ++e)
      if (!std::isfinite(x[e])) throw Error(kBadInput, "design vector contains NaN or Inf");
    p->p->set_design(x);
  });
}

int simp_get_design(simp_problem* p, double* x) {
  return guarded(p->err, [&] {
    use_device(p->device);
    p->p->get_design(x);
  });
}

int simp_evaluate(simp_problem* p, simp_evaluation* out, double* rho, double* dcp, double* dcx, double* dvx,
                  double* se, double* disp) {
  return guarded(p->err, [&] {
    use_device(p->device);
    GpuProblem& g = *p->p;
    const Evaluation ev = g.evaluate();
    if (out) {
      out->compliance = ev.compliance;
      out->volume = ev.volume;
      out->volume_fraction = ev.volume_fraction;
      out->linear_iterations = ev.linear_iterations;
      out->relres_max = ev.relres_max;
    }
    cudaStream_t s = g.amg.stream;
    const size_t ne = static_cast<size_t>(g.ne);
    if (rho) g.rho.download(rho, ne, s);
    if (dcp) g.dc_dphys.download(dcp, ne, s);
    if (dcx) g.dc_dx.download(dcx, ne, s);
    if (dvx) g.dv_dx.download(dvx, ne, s);
    if (se) g.se.download(se, ne, s);
    if (disp) {
      std::vector<double> uf(static_cast<size_t>(g.nfree) * g.d.nloads);
      g.u.download(uf.data(), uf.size(), s);
      const std::vector<i32> map = g.dof_map.to_host(s);
      for (int l = 0; l < g.d.nloads; ++l)
        for (i64 k = 0; k < g.ndof; ++k)
          disp[l * g.ndof + k] = map[k] >= 0 ? uf[static_cast<size_t>(l) * g.nfree + map[k]] : 0.0;
    }
    SIMP_CUDA(cudaStreamSynchronize(s));
  });
}

int simp_oc_update(simp_problem* p, int32_t apply, simp_oc_step* out, double* xnew) {
  return guarded(p->err, [&] {
    use_device(p->device);
    const OcStep st = p->p->oc_update(apply != 0, xnew);
    if (out) {
      out->lambda = st.lambda;
      out->achieved_volume = st.volume;
      out->max_change = st.max_change;
      out->bisections = st.bisections;
      out->volume_converged = st.converged ? 1 : 0;
    }
  });
}

int simp_mma_update(simp_problem* p, int32_t apply, simp_oc_step* out, double* xnew) {
  return guarded(p->err, [&] {
    use_device(p->device);
    const OcStep st = p->p->mma_update(apply != 0, xnew);
    if (out) {
      out->lambda = st.lambda;
      out->achieved_volume = st.volume;
      out->max_change = st.max_change;
      out->bisections = st.bisections;
      out->volume_converged = st.converged ? 1 : 0;
    }
  });
}

int simp_iterate(simp_problem* p, simp_iteration_record* rec) {
  return guarded(p->err, [&] {
    use_device(p->device);
    GpuProblem& g = *p->p;
    cudaEvent_t e0, e1;
    SIMP_CUDA(cudaEventCreate(&e0));
    SIMP_CUDA(cudaEventCreate(&e1));
    SIMP_CUDA(cudaEventRecord(e0, g.amg.stream));
    ++g.iteration;
    const Evaluation ev = g.evaluate();
    g.update_robust_target();
    const OcStep st = g.d.optimizer == 1 ? g.mma_update(true, nullptr) : g.oc_update(true, nullptr);
    SIMP_CUDA(cudaEventRecord(e1, g.amg.stream));
    SIMP_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    SIMP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rec) fill_record(g, ev, st, ms * 1e-3, rec);
    g.advance_beta(st.max_change);
  });
}

int simp_iterate_batch(simp_problem* const* problems, int32_t n, simp_iteration_record* records) {
  if (!problems || n < 1) {
    g_create_error = "simp_iterate_batch: no problems";
    return kBadInput;
  }
  const int dev = problems[0]->device;
  for (int i = 0; i < n; ++i)
    if (!problems[i] || problems[i]->device != dev) {
      g_create_error = "simp_iterate_batch: the problems must live on one device";
      return kBadInput;
    }
  for (int i = 0; i < n; ++i) problems[i]->err.clear();
  std::vector<int> codes(static_cast<size_t>(n), 0);
  auto record_error = [&](int i, int code, const std::string& msg) {
    problems[i]->err = msg;
    codes[static_cast<size_t>(i)] = code;
  };
  // fn(i) for every problem without an error, from a pool of host threads
  auto each = [&](auto&& fn) {
    const int workers = std::max(1, std::min<int>(n, static_cast<int>(std::thread::hardware_concurrency())));
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int k = 0; k < workers; ++k)
      pool.emplace_back([&] {
        cudaSetDevice(dev);
        for (int i = next++; i < n; i = next++) {
          if (codes[static_cast<size_t>(i)]) continue;
          try {
            fn(i);
          } catch (const Error& e) {
            record_error(i, e.code, e.what());
          } catch (const std::exception& e) {
            record_error(i, kBadInput, e.what());
          }
        }
      });
    for (auto& t : pool) t.join();
  };
  const auto t0 = std::chrono::steady_clock::now();
  each([&](int i) {
    GpuProblem& g = *problems[i]->p;
    ++g.iteration;
    g.evaluate_prepare();
    for (int l = 0; l < g.d.nloads; ++l) {
      SolveWork& w = g.amg.work(l);
      g.amg.ensure(w);
      g.start_load(l, w);
    }
    SIMP_CUDA(cudaStreamSynchronize(g.amg.stream));
  });
  std::vector<SolveTask> tasks;
  std::vector<std::pair<int, int>> owner;
  for (int i = 0; i < n; ++i) {
    if (codes[static_cast<size_t>(i)]) continue;
    GpuProblem& g = *problems[i]->p;
    for (int l = 0; l < g.d.nloads; ++l) {
      tasks.push_back(g.load_task(l, g.amg.work(l)));
      owner.emplace_back(i, l);
    }
  }
  std::vector<std::vector<GpuAmg::PcgResult>> res(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) res[static_cast<size_t>(i)].resize(static_cast<size_t>(problems[i]->p->d.nloads));
  try {
    use_device(dev);
    const std::vector<GpuAmg::TaskResult> tr = GpuAmg::solve_together(tasks);
    for (size_t k = 0; k < tr.size(); ++k) {
      const int i = owner[k].first, l = owner[k].second;
      if (tr[k].error_code) {
        if (!codes[static_cast<size_t>(i)]) record_error(i, tr[k].error_code, tr[k].error);
      } else {
        res[static_cast<size_t>(i)][static_cast<size_t>(l)] = tr[k].r;
      }
    }
  } catch (const Error& e) {
    for (int i = 0; i < n; ++i)
      if (!codes[static_cast<size_t>(i)]) record_error(i, e.code, e.what());
  }
  each([&](int i) {
    GpuProblem& g = *problems[i]->p;
    for (int l = 0; l < g.d.nloads; ++l) g.end_load(l, g.amg.work(l));
    const Evaluation ev = g.evaluate_finish(res[static_cast<size_t>(i)]);
    g.update_robust_target();
    const OcStep st = g.d.optimizer == 1 ? g.mma_update(true, nullptr) : g.oc_update(true, nullptr);
    SIMP_CUDA(cudaStreamSynchronize(g.amg.stream));
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (records) fill_record(g, ev, st, sec, &records[i]);
    g.advance_beta(st.max_change);
  });
  for (int i = 0; i < n; ++i)
    if (codes[static_cast<size_t>(i)]) return codes[static_cast<size_t>(i)];
  return kOk;
}

int simp_problem_stats(simp_problem* p, simp_amg_stats* s) {
  return guarded(p->err, [&] { fill_stats(p->p->amg, s); });
}

int simp_filter_forward(simp_problem* p, const double* x, double* y) {
  return guarded(p->err, [&] {
    use_device(p->device);
    GpuProblem& g = *p->p;
    const size_t ne = static_cast<size_t>(g.ne);
    DBuf<double> a, b(ne);
    a.upload(x, ne, g.amg.stream);
    g.filter_forward(a.p, b.p);
    b.download(y, ne, g.amg.stream);
    SIMP_CUDA(cudaStreamSynchronize(g.amg.stream));
  });
}

int simp_filter_adjoint(simp_problem* p, const double* v, double* gout) {
  return guarded(p->err, [&] {
    use_device(p->device);
    GpuProblem& g = *p->p;
    const size_t ne = static_cast<size_t>(g.ne);
    DBuf<double> a, b(ne);
    a.upload(v, ne, g.amg.stream);
    g.filter_adjoint(a.p, b.p);
    b.download(gout, ne, g.amg.stream);
    SIMP_CUDA(cudaStreamSynchronize(g.amg.stream));
  });
}

int simp_problem_kff(simp_problem* p, const double* scale, int32_t* rowptr, int32_t* col, double* val) {
  return guarded(p->err, [&] {
    use_device(p->device);
    GpuProblem& g = *p->p;
    Level& l0 = *g.amg.levels.front();
    if (val) {
      if (!scale) throw Error(kBadInput, "simp_problem_kff: values need element factors");
      DBuf<double> s;
      s.upload(scale, static_cast<size_t>(g.ne), g.amg.stream);
      g.assemble(s.p, true);
      l0.a.v64.download(val, static_cast<size_t>(l0.a.nnz), g.amg.stream);
      SIMP_CUDA(cudaStreamSynchronize(g.amg.stream));
    }
    if (rowptr) l0.a.ptr.download(rowptr, static_cast<size_t>(l0.n) + 1, g.amg.stream);
    if (col) l0.a.col.download(col, static_cast<size_t>(l0.a.nnz), g.amg.stream);
    SIMP_CUDA(cudaStreamSynchronize(g.amg.stream));
  });
}

int simp_element_stiffness(int32_t dim, double hx, double hy, double hz, double young, double poisson,
                           double thickness, double* ke) {
  return guarded(g_create_error, [&] {
    if (dim != 2 && dim != 3) throw Error(kBadInput, "dim must be 2 or 3");
    element_stiffness(dim, hx, hy, hz, young, poisson, thickness, ke);
  });
}

int simp_problem_apply_operator(simp_problem* p, const double* x, double* y) {
  return guarded(p->err, [&] {
    use_device(p->device);
    GpuAmg& amg = p->p->amg;
    if (!amg.ready()) throw Error(kBadInput, "the operator is assembled by the first evaluate");
    amg.spmv0(x, y);
  });
}

int simp_problem_apply_level0(simp_problem* p, const double* x, double* y) {
  return guarded(p->err, [&] {
    use_device(p->device);
    GpuAmg& amg = p->p->amg;
    if (!amg.ready()) throw Error(kBadInput, "the operator is assembled by the first evaluate");
    if (!x || !y) throw Error(kBadInput, "simp_problem_apply_level0: null vector");
    amg.spmv0_fast(x, y);
    amg.check_mf_status(amg.stream);
  });
}

int simp_problem_time_operator(simp_problem* p, int32_t reps, double* ms, double* bytes) {
  return guarded(p->err, [&] {
    use_device(p->device);
    double m = 0.0, b = 0.0;
    p->p->amg.time_operator(reps, &m, &b);
    if (ms) *ms = m;
    if (bytes) *bytes = b;
  });
}

int simp_filter_volume_noalloc(simp_problem* p, const double* x, double* rho, double* volume) {
  return guarded(p->err, [&] {
    use_device(p->device);
    filter_volume_noalloc(*p->p, x, rho, volume);
  });
}

int simp_projection_variants(simp_problem* p, double delta, simp_robust_record* record, double* eroded_density,
                             double* dilated_density) {
  return guarded(p->err, [&] {
    use_device(p->device);
    GpuProblem& g = *p->p;
    const double dl = delta > 0.0 ? delta : g.d.robust_delta;
    const GpuProblem::Variants v = g.projection_variants(dl, eroded_density, dilated_density);
    if (record) {
      record->eta_eroded = v.eta[0];
      record->eta_intermediate = v.eta[1];
      record->eta_dilated = v.eta[2];
      record->compliance_eroded = v.compliance[0];
      record->compliance_intermediate = v.compliance[1];
      record->compliance_dilated = v.compliance[2];
      record->volume_fraction_eroded = v.volume_fraction[0];
      record->volume_fraction_intermediate = v.volume_fraction[1];
      record->volume_fraction_dilated = v.volume_fraction[2];
      record->dilated_target_fraction = g.d.robust ? g.dilated_target / g.domain_volume : 0.0;
    }
  });
}

void simp_default_modal_options(simp_modal_options* o) {
  o->num_modes = 6;
  o->mass_type = 0;
  o->max_iterations = 200;
  o->tolerance = 1.0e-10;
  o->shift_factor = 0.0;
  o->rigid_body_ratio = 1.0e-10;
  o->residual_tolerance = 1.0e-6;
  o->warm_start = 1;
  o->density = 1.0;
  o->element_mass = nullptr;
  o->concurrent_solves = 4;
}

int simp_modal(simp_problem* p, const simp_modal_options* options, const double* stiffness_scale,
               const double* mass_scale, double* eigenvalues, double* frequencies_hz, double* residuals,
               double* mass_fraction, double* mode_shapes, simp_modal_info* info) {
  return guarded(p->err, [&] {
    use_device(p->device);
    if (!options) throw Error(kBadInput, "simp_modal needs options");
    GpuProblem& g = *p->p;
    ModalOptions o;
    o.num_modes = options->num_modes;
    o.mass_type = options->mass_type;
    o.max_iterations = options->max_iterations;
    o.tolerance = options->tolerance;
    o.shift_factor = options->shift_factor;
    o.rigid_body_ratio = options->rigid_body_ratio;
    o.residual_tolerance = options->residual_tolerance;
    o.warm_start = options->warm_start != 0;
    o.density = options->density;
    o.concurrent_solves = options->concurrent_solves;
    if (options->element_mass) {
      const int ed = g.d.dim == 3 ? 24 : 8;
      o.element_mass.assign(options->element_mass, options->element_mass + ed * ed);
    }
    p->modal_warnings.clear();
    const ModalResult r = solve_modal(g, o, stiffness_scale, mass_scale, mode_shapes != nullptr);
    p->modal_warnings = r.warnings;
    const int m = static_cast<int>(r.eigenvalues.size());
    constexpr double two_pi = 6.283185307179586476925286766559;
    for (int i = 0; i < m; ++i) {
      if (eigenvalues) eigenvalues[i] = r.eigenvalues[i];
      if (frequencies_hz) frequencies_hz[i] = std::sqrt(std::max(r.eigenvalues[i], 0.0)) / two_pi;
      if (residuals) residuals[i] = r.residuals[i];
      if (mass_fraction) mass_fraction[i] = r.mass_fraction[i];
    }
    if (mode_shapes) std::copy(r.shapes.begin(), r.shapes.end(), mode_shapes);
    if (info) {
      info->num_modes = m;
      info->iterations = r.iterations;
      info->subspace_size = r.subspace_size;
      info->converged = r.converged ? 1 : 0;
      info->linear_iterations = r.linear_iterations;
      info->final_change = r.final_change;
      info->total_mass = r.total_mass;
      info->num_warnings = static_cast<int32_t>(r.warnings.size());
    }
  });
}

const char* simp_modal_warning(simp_problem* p, int32_t k) {
  if (!p || k < 0 || k >= static_cast<int32_t>(p->modal_warnings.size())) return nullptr;
  return p->modal_warnings[static_cast<size_t>(k)].c_str();
}

void simp_default_buckling_options(simp_buckling_options* o) {
  o->num_modes = 4;
  o->max_iterations = 400;
  o->tolerance = 1.0e-8;
  o->residual_tolerance = 1.0e-6;
  o->young = 0.0;
  o->poisson = 0.0;
  o->transform = 0;
  o->concurrent_solves = 4;
  o->shift_hint = 0.0;
}

int simp_buckling(simp_problem* p, const simp_buckling_options* options, int32_t load_case,
                  const double* stiffness_scale, const double* stress_scale, const uint8_t* solid_mask,
                  const double* start_subspace, int32_t start_cols, double* load_factors, double* residuals,
                  double* solid_energy_fraction, double* mode_shapes, double* subspace, simp_buckling_info* info) {
  return guarded(p->err, [&] {
    use_device(p->device);
    if (!options) throw Error(kBadInput, "simp_buckling needs options");
    BucklingOptions o;
    o.num_modes = options->num_modes;
    o.max_iterations = options->max_iterations;
    o.tolerance = options->tolerance;
    o.residual_tolerance = options->residual_tolerance;
    o.young = options->young;
    o.poisson = options->poisson;
    o.transform = options->transform;
    o.concurrent_solves = options->concurrent_solves;
    o.shift_hint = options->shift_hint;
    p->buckling_warnings.clear();
    const BucklingResult r = solve_buckling(*p->p, o, load_case, stiffness_scale, stress_scale, solid_mask,
                                            start_subspace, start_cols, mode_shapes != nullptr);
    p->buckling_warnings = r.warnings;
    const int m = static_cast<int>(r.load_factors.size());
    for (int i = 0; i < m; ++i) {
      if (load_factors) load_factors[i] = r.load_factors[i];
      if (residuals) residuals[i] = r.residuals[i];
      if (solid_energy_fraction) solid_energy_fraction[i] = r.solid_fraction[i];
    }
    if (mode_shapes) std::copy(r.shapes.begin(), r.shapes.end(), mode_shapes);
    if (subspace) std::copy(r.subspace.begin(), r.subspace.end(), subspace);
    if (info) {
      info->num_modes = m;
      info->iterations = r.iterations;
      info->subspace_size = r.subspace_size;
      info->converged = r.converged ? 1 : 0;
      info->no_positive_load_factor = r.no_positive ? 1 : 0;
      info->subspace_cols = r.subspace_cols;
      info->linear_iterations = r.linear_iterations;
      info->final_change = r.final_change;
      info->num_warnings = static_cast<int32_t>(r.warnings.size());
      info->transformed = r.transformed ? 1 : 0;
      info->sigma = r.sigma;
      info->factorizations = r.factorizations;
    }
  });
}

const char* simp_buckling_warning(simp_problem* p, int32_t k) {
  if (!p || k < 0 || k >= static_cast<int32_t>(p->buckling_warnings.size())) return nullptr;
  return p->buckling_warnings[static_cast<size_t>(k)].c_str();
}

int simp_element_mass(int32_t dim, double hx, double hy, double hz, double density, double thickness,
                      double* me) {
  return guarded(g_create_error, [&] {
    if (dim != 2 && dim != 3) throw Error(kBadInput, "dim must be 2 or 3");
    if (!(density > 0.0)) throw Error(kBadInput, "mass assembly requires a positive density");
    element_mass(dim, hx, hy, hz, density, thickness, me);
  });
}

int64_t simp_kernel_launches(void) { return g_launches.load(); }

}  // extern "C"

// ---- the displacement surrogate (surrogate_net.cu) ---------------------
struct simp_surrogate {
  std::unique_ptr<sg::Surrogate> s;
  int device = 0;
};

namespace {
template <class F>
int sg_guarded(F&& f) {
  try {
    f();
    return kOk;
  } catch (const Error& e) {
    sg::last_error() = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    sg::last_error() = "out of host memory";
    return kBadInput;
  } catch (const std::exception& e) {
    sg::last_error() = e.what();
    return kBadInput;
  }
}
}  // namespace

extern "C" {

int simp_surrogate_create(int32_t device, uint64_t seed, simp_surrogate** out) {
  return sg_guarded([&] {
    if (!out) throw Error(kBadInput, "simp_surrogate_create: out is NULL");
    use_device(device);
    std::unique_ptr<simp_surrogate> h(new simp_surrogate());
    h->device = device;
    h->s.reset(new sg::Surrogate(seed));
    *out = h.release();
  });
}

void simp_surrogate_destroy(simp_surrogate* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  delete s;
}

int simp_surrogate_num_params(simp_surrogate* s, int64_t* n) {
  return sg_guarded([&] { *n = static_cast<int64_t>(s->s->net.nparams); });
}

int simp_surrogate_get_params(simp_surrogate* s, float* params) {
  return sg_guarded([&] {
    use_device(s->device);
    s->s->net.get_params(params);
  });
}

int simp_surrogate_set_params(simp_surrogate* s, const float* params) {
  return sg_guarded([&] {
    use_device(s->device);
    s->s->net.set_params(params);
  });
}

int simp_surrogate_add_sample(simp_surrogate* s, simp_problem* p, int32_t load_case) {
  return sg_guarded([&] {
    use_device(s->device);
    if (load_case < 0 || load_case >= p->p->d.nloads) throw Error(kBadInput, "load case out of range");
    s->s->add_sample(*p->p, load_case);
  });
}

int simp_surrogate_num_samples(simp_surrogate* s, int32_t* n) {
  return sg_guarded([&] { *n = static_cast<int32_t>(s->s->samples.size()); });
}

int simp_surrogate_train(simp_surrogate* s, int32_t epochs, double learning_rate, int32_t batch, uint64_t seed,
                         double* epoch_losses) {
  return sg_guarded([&] {
    use_device(s->device);
    if (epochs < 1 || batch < 1 || !(learning_rate > 0.0)) throw Error(kBadInput, "simp_surrogate_train: bad options");
    const size_t before = s->s->losses.size();
    s->s->train(epochs, learning_rate, batch, seed);
    if (epoch_losses)
      for (int e = 0; e < epochs; ++e) epoch_losses[e] = s->s->losses[before + static_cast<size_t>(e)];
  });
}

int simp_surrogate_predict(simp_surrogate* s, simp_problem* p, int32_t load_case, double* u_device) {
  return sg_guarded([&] {
    use_device(s->device);
    if (load_case < 0 || load_case >= p->p->d.nloads) throw Error(kBadInput, "load case out of range");
    if (!u_device) throw Error(kBadInput, "simp_surrogate_predict: NULL output");
    s->s->predict(*p->p, load_case, u_device);
  });
}

int simp_surrogate_forward(simp_surrogate* s, int32_t nx, int32_t ny, int32_t nz, const void* input_device,
                           float* output_device) {
  return sg_guarded([&] {
    use_device(s->device);
    if (nx < 2 || ny < 2 || nz < 2) throw Error(kBadInput, "simp_surrogate_forward: at least 2 nodes per axis");
    sg::Net& net = s->s->net;
    net.shape(nx, ny, nz);
    const size_t nodes = static_cast<size_t>(nx) * ny * nz;
    SIMP_CUDA(cudaMemcpyAsync(net.in16.p, input_device, nodes * 16 * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice,
                              net.stream));
    net.forward();
    SIMP_CUDA(cudaMemcpyAsync(output_device, net.out.p, nodes * 3 * sizeof(float), cudaMemcpyDeviceToDevice,
                              net.stream));
    SIMP_CUDA(cudaStreamSynchronize(net.stream));
    net.check_status();
  });
}

int simp_surrogate_loss_gradient(simp_surrogate* s, int32_t nx, int32_t ny, int32_t nz, const void* input_device,
                                  const void* target_device, const uint8_t* mask_device, int64_t count, double* loss,
                                  float* gradient) {
  return sg_guarded([&] {
    use_device(s->device);
    if (nx < 2 || ny < 2 || nz < 2 || count < 1) throw Error(kBadInput, "simp_surrogate_loss_gradient: bad sizes");
    sg::Net& net = s->s->net;
    net.shape(nx, ny, nz);
    const size_t nodes = static_cast<size_t>(nx) * ny * nz;
    SIMP_CUDA(cudaMemcpyAsync(net.in16.p, input_device, nodes * 16 * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice,
                              net.stream));
    net.grad.zero(net.stream);
    net.forward();
    *loss = net.loss(static_cast<const __nv_bfloat16*>(target_device), mask_device, count);
    net.backward();
    SIMP_CUDA(cudaMemcpyAsync(gradient, net.grad.p, sizeof(float) * net.nparams, cudaMemcpyDeviceToHost, net.stream));
    net.grad.zero(net.stream);
    SIMP_CUDA(cudaStreamSynchronize(net.stream));
    net.check_status();
  });
}

int simp_problem_set_surrogate(simp_problem* p, simp_surrogate* s) {
  return guarded(p->err, [&] {
    if (s && s->device != p->device) throw Error(kBadInput, "the surrogate lives on another device");
    p->p->surrogate = s ? s->s.get() : nullptr;
  });
}

int simp_problem_learned_seconds(simp_problem* p, double* seconds) {
  return guarded(p->err, [&] { *seconds = p->p->learned_seconds; });
}

}  // extern "C"

extern "C" {

void simp_autotune_enable(int32_t on) { tune_set_enabled(on != 0); }

int simp_autotune_set(const char* key, int32_t variant) {
  if (!key || variant < 0) return kBadInput;
  tune_set(key, variant);
  return kOk;
}

int simp_autotune_report(char* buf, int64_t size, int64_t* needed) {
  std::ostringstream os;
  for (const TuneRecord& r : tune_records()) {
    os << r.key << ' ' << r.chosen;
    for (double ms : r.ms) os << ' ' << ms;
    os << '\n';
  }
  const std::string text = os.str();
  if (needed) *needed = static_cast<int64_t>(text.size()) + 1;
  if (buf && size > 0) {
    const size_t n = std::min(static_cast<size_t>(size - 1), text.size());
    std::memcpy(buf, text.data(), n);
    buf[n] = '\0';
  }
  return kOk;
}

}  // extern "C"
