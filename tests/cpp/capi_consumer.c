/* A plain C99 consumer of include/otfem_gpu.h: one tet, one reference step.
 * Shows that the boundary is a C ABI (no C++ or CUDA types in its
 * signatures).  Used by tests/test_dropin_cpp.py. */
#include <stdio.h>

#include "otfem_gpu.h"

int main(void) {
  int32_t tets[4] = {0, 1, 2, 3};
  double coord[12] = {0, 0, 0, 0.1, 0, 0, 0, 0.1, 0, 0, 0, 0.1};
  uint8_t fixed[4] = {1, 0, 0, 0};
  otfem_mesh_desc d = {4, 1, tets, coord, NULL, fixed};
  otfem_handle h = NULL;
  double f[12] = {0};
  double x[12];
  int rc = otfem_create(&d, NULL, &h);
  if (rc != OTFEM_OK) {
    printf("create: %d %s\n", rc, otfem_last_error());
    return 1;
  }
  rc = otfem_init(h, 5e5, 0.33, 1000.0, 1e30, 0.0, 0.0);
  f[4] = -9.81;
  if (rc == OTFEM_OK) rc = otfem_set_nodes(h, OTFEM_F_EXTERNAL, f, 12);
  if (rc == OTFEM_OK) rc = otfem_simulate(h, 0.01, 1);
  if (rc == OTFEM_OK) rc = otfem_get_nodes(h, OTFEM_COORD, x, 12);
  if (rc != OTFEM_OK) {
    printf("error %d: %s\n", rc, otfem_last_error());
    return 1;
  }
  printf("%.17g %.17g %.17g\n", x[3], x[4], x[5]);
  otfem_destroy(h);
  return 0;
}
