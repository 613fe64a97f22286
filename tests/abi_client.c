/* A plain C99 caller of include/simp_gpu.h, linked against libsimp_gb300.so.
 *
 * It drives the LinearSolver boundary the way a C or cgo/ctypes caller would:
 * simp_default_options -> simp_ctx_create -> simp_set_layout ->
 * simp_factorize -> simp_solve -> simp_stats -> simp_ctx_destroy, and reports
 * a failed call by its status code (the process exit status) and the text of
 * simp_last_error, read after the failing call and before the next one.
 *
 *   abi_client bad-options
 *       simp_ctx_create with an out-of-range coarse_size: must fail with
 *       SIMP_BAD_INPUT before any device call (runs without a GPU).
 *   abi_client solve <system.bin> <solution.bin> [max_iterations]
 *       reads a system written by the tests (little-endian):
 *         int32 dim, n, num_nodes; int64 nnz;
 *         double coords[dim * num_nodes]; int32 unknowns[n];
 *         int32 rowptr[n + 1]; int32 colidx[nnz]; double values[nnz];
 *         double rhs[n]; double rtol
 *       and writes: int32 status, iterations, num_levels; double relres,
 *       operator_complexity; double x[n].
 */
#include "simp_gpu.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static int read_all(FILE* f, void* p, size_t size, size_t count) {
  return fread(p, size, count, f) == count;
}

static int bad_options(void) {
  simp_solver_options o;
  simp_ctx* ctx = NULL;
  int code;
  simp_default_options(&o);
  o.coarse_size = 0;
  code = simp_ctx_create(&o, &ctx);
  if (code != SIMP_BAD_INPUT || ctx != NULL) {
    fprintf(stderr, "expected SIMP_BAD_INPUT, got %d\n", code);
    return 100;
  }
  /* the message of a failed create is read with a NULL context */
  printf("status %d: %s\n", code, simp_last_error(NULL));
  return strlen(simp_last_error(NULL)) > 0 ? code : 101;
}

static int solve(const char* in_path, const char* out_path, int max_iterations) {
  FILE* f = fopen(in_path, "rb");
  int32_t dim, n, nodes, status = SIMP_OK, iterations = 0;
  int64_t nnz;
  double *coords, *values, *rhs, *x, rtol, relres = 0.0;
  int32_t *unknowns, *rowptr, *colidx;
  simp_solver_options o;
  simp_ctx* ctx = NULL;
  simp_amg_stats st;
  if (!f) return 102;
  if (!read_all(f, &dim, 4, 1) || !read_all(f, &n, 4, 1) || !read_all(f, &nodes, 4, 1) ||
      !read_all(f, &nnz, 8, 1))
    return 103;
  coords = malloc(sizeof(double) * (size_t)dim * nodes);
  unknowns = malloc(sizeof(int32_t) * (size_t)n);
  rowptr = malloc(sizeof(int32_t) * (size_t)(n + 1));
  colidx = malloc(sizeof(int32_t) * (size_t)nnz);
  values = malloc(sizeof(double) * (size_t)nnz);
  rhs = malloc(sizeof(double) * (size_t)n);
  x = calloc((size_t)n, sizeof(double));
  if (!read_all(f, coords, 8, (size_t)dim * nodes) || !read_all(f, unknowns, 4, (size_t)n) ||
      !read_all(f, rowptr, 4, (size_t)n + 1) || !read_all(f, colidx, 4, (size_t)nnz) ||
      !read_all(f, values, 8, (size_t)nnz) || !read_all(f, rhs, 8, (size_t)n) || !read_all(f, &rtol, 8, 1))
    return 104;
  fclose(f);

  simp_default_options(&o);
  o.iterative_tolerance = rtol;
  o.max_iterations = max_iterations;
  memset(&st, 0, sizeof(st));
  status = simp_ctx_create(&o, &ctx);
  if (status != SIMP_OK) {
    fprintf(stderr, "simp_ctx_create: %s\n", simp_last_error(NULL));
  } else {
    status = simp_set_layout(ctx, dim, dim, coords, nodes, unknowns, n);
    if (status == SIMP_OK) status = simp_factorize(ctx, n, rowptr, colidx, values);
    if (status == SIMP_OK) status = simp_solve(ctx, 1, rhs, NULL, x, &iterations, &relres);
    if (status != SIMP_OK) {
      /* the message stays valid until the next call on this context */
      const char* msg = simp_last_error(ctx);
      fprintf(stderr, "status %d: %s\n", status, msg);
      printf("%s\n", msg);
    } else if (simp_stats(ctx, &st) != SIMP_OK) {
      status = 105;
    }
    simp_ctx_destroy(ctx);
  }
  f = fopen(out_path, "wb");
  if (!f) return 106;
  fwrite(&status, 4, 1, f);
  fwrite(&iterations, 4, 1, f);
  fwrite(&st.num_levels, 4, 1, f);
  fwrite(&relres, 8, 1, f);
  fwrite(&st.operator_complexity, 8, 1, f);
  fwrite(x, 8, (size_t)n, f);
  fclose(f);
  free(coords);
  free(unknowns);
  free(rowptr);
  free(colidx);
  free(values);
  free(rhs);
  free(x);
  return status;
}

int main(int argc, char** argv) {
  if (argc >= 2 && strcmp(argv[1], "bad-options") == 0) return bad_options();
  if (argc >= 4 && strcmp(argv[1], "solve") == 0)
    return solve(argv[2], argv[3], argc >= 5 ? atoi(argv[4]) : 0);
  fprintf(stderr, "usage: abi_client bad-options | solve <system.bin> <solution.bin> [max_iterations]\n");
  return 2;
}
