/* A compiled host program on the C ABI, as the Fortran driver of iModel's
 * swm_tests would use it (src/swm.f90:238-370): build the grid, create a
 * handle, run the time loop one imodel_swm_step per RK4 step on host
 * arrays (swm.f90:249, ode_rk4), print the diagnostics every `every`
 * steps (swm.f90:293-322), write the final state.
 *
 *   swm_driver level precision nsteps dt every h_in u_in h_out u_out [gpu]
 *
 * precision 0 = FP64, 1 = FP32; the state files hold nv and ne doubles in
 * the grid's order; gpu = 1 builds the grid with imodel_mesh_build_gpu. */
#include <stdio.h>
#include <stdlib.h>

#include "imodel_mesh.h"
#include "imodel_swm.h"

static int read_doubles(const char *path, double *x, size_t n) {
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  const size_t got = fread(x, sizeof(double), n, f);
  fclose(f);
  return got == n ? 0 : 1;
}

static int write_doubles(const char *path, const double *x, size_t n) {
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  const size_t put = fwrite(x, sizeof(double), n, f);
  fclose(f);
  return put == n ? 0 : 1;
}

int main(int argc, char **argv) {
  if (argc != 10 && argc != 11) {
    fprintf(stderr, "usage: %s level precision nsteps dt every h_in u_in h_out u_out [gpu]\n",
            argv[0]);
    return 2;
  }
  const int level = atoi(argv[1]), precision = atoi(argv[2]), nsteps = atoi(argv[3]);
  const double dt = atof(argv[4]);
  const int every = atoi(argv[5]);
  const int gpu_grid = argc == 11 && atoi(argv[10]) == 1;
  void *grid = NULL;
  int rc = gpu_grid ? imodel_mesh_build_gpu(level, 0, 0, &grid) : imodel_mesh_build(level, 0, 0, &grid);
  if (rc) {
    fprintf(stderr, "grid build failed: %d\n", rc);
    return 3;
  }
  imodel_swm_mesh m;
  imodel_mesh_view(grid, &m);
  double *h = malloc(sizeof(double) * (size_t)m.nv), *u = malloc(sizeof(double) * (size_t)m.ne);
  if (!h || !u || read_doubles(argv[6], h, (size_t)m.nv) || read_doubles(argv[7], u, (size_t)m.ne)) {
    fprintf(stderr, "cannot read the initial state\n");
    return 4;
  }
  imodel_swm_opts o = {0};
  o.precision = precision;
  o.testcase = 2;
  void *swm = NULL;
  rc = imodel_swm_create(&m, &o, &swm);
  if (rc) {
    fprintf(stderr, "create failed: %d %s\n", rc, imodel_swm_last_error(swm));
    imodel_swm_destroy(swm);
    return 5;
  }
  for (int n = 1; n <= nsteps; ++n) {
    rc = imodel_swm_step(swm, h, u, dt, 1);
    if (rc) {
      fprintf(stderr, "step %d failed: %d %s\n", n, rc, imodel_swm_last_error(swm));
      imodel_swm_destroy(swm);
      return 6;
    }
    if (every > 0 && n % every == 0) {
      imodel_swm_diag d;
      rc = imodel_swm_diagnostics(swm, &d);
      if (rc) return 7;
      printf("step %d mass %.17g tenergy %.17g pot_enstrophy %.17g\n", n, d.mass, d.tenergy,
             d.pot_enstrophy);
    }
  }
  rc = write_doubles(argv[8], h, (size_t)m.nv) || write_doubles(argv[9], u, (size_t)m.ne);
  imodel_swm_destroy(swm);
  imodel_mesh_free(grid);
  free(h);
  free(u);
  return rc ? 8 : 0;
}
