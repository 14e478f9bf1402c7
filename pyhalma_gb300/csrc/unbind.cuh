// Device-array entry points shared between translation units (no staging, no locking).
#pragma once
#include "common.cuh"

namespace halma {

// Optional measurement state (halma_set_profiling): CUDA events recorded on the launching
// stream around every pair-kernel launch (captured into the pass graph as event nodes) and
// the pair count of each pass, read back at the end of the call.
struct Profile {
    bool enabled = false;
    std::vector<cudaEvent_t> ev0, evm, ev1;   // per pass: before, between and after the pair kernels
    struct Pass {
        double pairs, ms, sym_pairs;   // sym_pairs: the part done by the symmetric block kernel
        double sym_ms;                 // time of the symmetric block kernel alone (0 when absent)
    };
    std::vector<Pass> passes;
    double fof_ms = 0, unbind_ms = 0;
    // FoF stages of the last plain FoF (keys, sort, records, cells, items, links, labels,
    // groups), milliseconds between events recorded on the launching stream
    static constexpr int kFofStages = 8;
    cudaEvent_t fev[kFofStages + 1] = {};
    double fof_stage_ms[kFofStages] = {};
    int ensure_events(int k);
    int fof_mark(int stage, cudaStream_t st);   // records fev[stage] when profiling (0..kFofStages)
};
Profile &profile();

// Tile shape per halo size class for the batched pair kernel: a halo with nb bound
// particles uses T = t[c] targets per lane for the first class c with nb <= upper[c].
constexpr int kMaxTileClasses = 8;
struct TileTable {
    int n;
    int upper[kMaxTileClasses];
    int t[kMaxTileClasses];
    int slice;   // source slots per work item (multiple of 32)
};
TileTable tile_table();

int bbox_device(int n, const double *x, const double *y, const double *z, double bb[7], cudaStream_t st);
int fof_device(int n, const double *x, const double *y, const double *z, double ll, int *labels,
               int64_t *n_groups, cudaStream_t st);
int fof_groups_device(int n, const int *labels, int minp, int64_t *offsets, int *members,
                      int64_t *n_groups, int64_t *n_members, cudaStream_t st);
int fof_segmented_device(int n, int nseg, const int64_t *off, const double *x, const double *y, const double *z,
                         double ll, int *labels, int64_t *n_groups, cudaStream_t st);
int reductions_device(int64_t n, int nh, const int64_t *off, const double *x, const double *y, const double *z,
                      const double *vx, const double *vy, const double *vz, const double *m,
                      const unsigned char *mask, const double *about, double *out, cudaStream_t st);
int sym_block_count(int nb);
int sym_self_potential_device(const float4 *pk, int nb, float eps2, float2 *part, void *scratch, cudaStream_t st);
int unbind_device(int64_t n, int nh, const int64_t *d_off, const int64_t *h_off, const double *x,
                  const double *y, const double *z, const double *vx, const double *vy,
                  const double *vz, const double *m, const halma_unbind_params &p,
                  unsigned char *bound, double *phi_out, double *halo_out, cudaStream_t st,
                  cudaEvent_t vel_ready = nullptr);

}  // namespace halma
