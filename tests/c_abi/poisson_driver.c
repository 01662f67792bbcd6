/* A C driver of the C-ABI: the steps of tutorial_01's serial Poisson driver (mesh, FE space
 * with strong Dirichlet conditions, affine operator, CG with Jacobi) through
 * include/fempar_gpu.h only.  It is what a Fortran shim calls through ISO_C_BINDING.
 * Usage: poisson_driver [n] [order] [rtol] [solution_file]; prints one line with the dof
 * count, the CG iterations, the final residual estimate and the first upper-CSR row length,
 * and writes the solution (num_free doubles, native byte order) when a file is given. */
#include <stdio.h>
#include <stdlib.h>

#include "fempar_gpu.h"

#define CHECK(call)                                                                   \
  do {                                                                                \
    fg_status s_ = (call);                                                            \
    if (s_ != FG_OK && s_ != FG_ERR_NOT_CONVERGED) {                                  \
      fprintf(stderr, "%s: %s (%s)\n", #call, fg_status_string(s_), fg_last_error()); \
      return 1;                                                                       \
    }                                                                                 \
  } while (0)

int main(int argc, char** argv) {
  const int n = argc > 1 ? atoi(argv[1]) : 8, order = argc > 2 ? atoi(argv[2]) : 2;
  const double rtol = argc > 3 ? atof(argv[3]) : 1e-8;
  const char* out_path = argc > 4 ? argv[4] : NULL;
  fg_ctx* ctx = NULL;
  fg_mesh* mesh = NULL;
  fg_space* space = NULL;
  fg_system* sys = NULL;
  CHECK(fg_ctx_create(0, 0, &ctx));
  const int32_t cells[3] = {n, n, n};
  const double limits[6] = {0.0, 1.0, 0.0, 1.0, 0.0, 1.0};
  CHECK(fg_mesh_create_structured(ctx, 3, cells, limits, NULL, &mesh));
  int32_t ids[26];
  for (int i = 0; i < 26; ++i) ids[i] = i + 1; /* every boundary set of the generator */
  CHECK(fg_space_create(mesh, order, 1, ids, 26, &space));
  fg_space_info info;
  CHECK(fg_space_get_info(space, &info));
  fg_integrand g;
  fg_integrand_default(&g);
  g.kind = FG_POISSON;
  g.source_fn = FG_FN_SHARP_WAVE;
  g.boundary_fn = FG_FN_SHARP_WAVE;
  const double sharp[5] = {50.0, 0.7, -0.05, -0.05, -0.05};
  for (int i = 0; i < 5; ++i) g.fn_param[i] = sharp[i];
  CHECK(fg_assemble(space, &g, &sys));
  fg_solver_params prm;
  fg_solver_params_default(&prm);
  prm.precond = FG_PREC_JACOBI;
  prm.rtol = rtol;
  prm.max_iters = 100000;
  double* x = (double*)calloc((size_t)info.num_free, sizeof(double));
  fg_solve_info sinfo;
  CHECK(fg_solve(sys, &prm, NULL, NULL, x, &sinfo));
  int64_t* irp = (int64_t*)malloc(sizeof(int64_t) * (size_t)(info.num_free + 1));
  int32_t* ja = (int32_t*)malloc(sizeof(int32_t) * (size_t)(info.nnz_upper > 0 ? info.nnz_upper : 1));
  double* val = (double*)malloc(sizeof(double) * (size_t)(info.nnz_upper > 0 ? info.nnz_upper : 1));
  CHECK(fg_system_export_csr(sys, 1, 1, irp, ja, val));
  printf("dofs %lld iterations %d converged %d residual %.3e first_row %lld\n", (long long)info.num_free,
         sinfo.iterations, sinfo.converged, sinfo.error_estimate,
         (long long)(info.num_free > 0 ? irp[1] - irp[0] : 0));
  if (out_path) {
    FILE* f = fopen(out_path, "wb");
    if (!f || fwrite(x, sizeof(double), (size_t)info.num_free, f) != (size_t)info.num_free) {
      fprintf(stderr, "cannot write %s\n", out_path);
      return 1;
    }
    fclose(f);
  }
  free(x);
  free(irp);
  free(ja);
  free(val);
  fg_system_destroy(sys);
  fg_space_destroy(space);
  fg_mesh_destroy(mesh);
  fg_ctx_destroy(ctx);
  return 0;
}
