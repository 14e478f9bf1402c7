// Device-array entry points shared between translation units (no staging, no locking).
#pragma once
#include "common.cuh"

namespace halma {

int fof_device(int n, const double *x, const double *y, const double *z, double ll, int *labels,
               int64_t *n_groups, cudaStream_t st);
int fof_groups_device(int n, const int *labels, int minp, int64_t *offsets, int *members,
                      int64_t *n_groups, int64_t *n_members, cudaStream_t st);
int unbind_device(int64_t n, int nh, const int64_t *d_off, const int64_t *h_off, const double *x,
                  const double *y, const double *z, const double *vx, const double *vy,
                  const double *vz, const double *m, const halma_unbind_params &p,
                  unsigned char *bound, double *phi_out, double *halo_out, cudaStream_t st);

}  // namespace halma
