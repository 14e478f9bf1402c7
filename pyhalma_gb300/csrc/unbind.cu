// Batched iterative unbinding of thousands of haloes, and the plain FP64 per-halo path.
//
// The single pass is pyHALMA's escape cut (python_scripts/halo_properties.py:282-361):
//     E_i = 1/2 |v_i - v_bulk|^2 - G * factor_v^2 * phi_i,   bound iff E_i <= 0
// repeated until a pass removes nothing.  Before the first pass:
//   reduce  - per halo, FP64 mass, centre of mass and bulk velocity;
//   pack    - members re-centred on their halo's centre, float4 (x, y, z, m), padded to a
//             multiple of 32 with zero-mass far points (halo-contiguous slots).
// Every pass over all active haloes is then five kernels:
//   items   - the implicit work list: per halo, (target tile of 32*T) x (source slice) items,
//             biggest haloes first, and the energy segments of the pass;
//   pairs   - persistent kernel: warps take items from an atomic counter, stream the slice's
//             sources through a per-warp shared-memory chunk, two sources per f32x2
//             instruction, 32-term FP32 partials folded into a TwoSum-compensated
//             accumulator; the self pair is skipped by slot index;
//   energy / compact / finalize - FP64 energy and sign test, survivors compacted into the
//             other packed buffer, next pass's FP64 centre and bulk velocity; a halo whose pass
//             removed nothing becomes inactive and costs nothing later.
// All passes are captured once into a CUDA graph and replayed (cached by shape).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "pair_math.cuh"
#include "sort.cuh"
#include "unbind.cuh"

namespace halma {

namespace {

constexpr int kUbWarps = 8;
constexpr float kFar = 3.0e30f;

struct HaloState {   // per halo, FP64 unless stated
    double M, cx, cy, cz, vx, vy, vz, ekin, epot;
    // FP32 path: sums of m x and m v over the bound set, kept up to date by subtracting each
    // pass's removed particles; the bulk velocity at packing (packed velocities are relative
    // to it) and the current bulk velocity relative to it in FP32
    double sx, sy, sz, px, py, pz, v0x, v0y, v0z;
    float wx, wy, wz;
    int nb, active, iter, removed, nrem;   // nrem: removed by the last pass (next pass's sources)
    int nprev;                             // slots the last pass examined (nb before its cut)
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide FP64 sums of NV values written to out[0..NV) (fixed association: warp tree,
// then the warps in order).
template <int NV>
__device__ __forceinline__ void block_sum_store(const double (&v)[NV], double (*sh)[32], double *out) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = warp_sum(v[q]);
        if (lane == 0) sh[q][w] = s;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = lane < nw ? sh[q][lane] : 0.0;
            s = warp_sum(s);
            if (lane == 0) out[q] = s;
        }
    }
}

__global__ void ub_init_kernel(int64_t n, unsigned char *bound, int nh, HaloState *hs) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        bound[i] = 1;
    for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
        HaloState s{};
        s.active = 1;
        hs[h] = s;
    }
}

// Member chunks: every halo's CSR range is cut into chunks of kSeg members, chunk c covering
// members off[h] + (c - cstart[h]) * kSeg onward of halo h = chunk_h[c] (laid out on the host),
// so a large halo is spread over many blocks.
constexpr int kSeg = 1024;
constexpr int kSegThreads = 256;
constexpr int kSegPer = kSeg / kSegThreads;
constexpr int kRedSums = 8;   // M, Mx, My, Mz, Mvx, Mvy, Mvz, count

// Per member chunk of an active halo (or of every halo with force): FP64 sums over its bound
// members.  FP64 is slow on this GPU, so the block's partials are combined by a few threads
// in shared memory rather than by warp trees (fixed association: per thread in member order,
// then per value four runs of 64 threads, then the four runs in order).  PART selects the
// sums written: 0 all, 1 mass, mass-weighted positions and count (the velocities are not
// read), 2 the mass-weighted velocities; each sum is formed the same way in every mode, so
// modes 1 then 2 write exactly what mode 0 writes.
__host__ __device__ constexpr bool red_wants(int part, int k) { return part == 0 || (part == 1 ? (k < 4 || k == 7) : (k >= 4 && k < 7)); }

template <int PART>
__global__ void __launch_bounds__(kSegThreads) ub_reduce_seg_kernel(
    const int64_t *__restrict__ off, const int *__restrict__ cstart, const int *__restrict__ chunk_h,
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
    const double *__restrict__ vx, const double *__restrict__ vy, const double *__restrict__ vz,
    const double *__restrict__ m, const unsigned char *__restrict__ bound, const HaloState *__restrict__ hs,
    int force, double *__restrict__ part) {
    const int c = blockIdx.x;
    const int h = chunk_h[c];
    if (!force && !hs[h].active) return;
    __shared__ double sh[kRedSums - 1][kSegThreads];
    __shared__ double q4[kRedSums - 1][4];
    const int64_t b = off[h] + (int64_t)(c - cstart[h]) * kSeg;
    const int64_t e = min(off[h + 1], b + kSeg);
    double v[kRedSums - 1] = {0, 0, 0, 0, 0, 0, 0};
    int count = 0;
    // all loads of the thread's members are issued before any is used; members outside the
    // chunk read member b and are skipped
    bool use[kSegPer];
    double f[kSegPer][7];
#pragma unroll
    for (int j = 0; j < kSegPer; ++j) {
        const int64_t i = b + j * kSegThreads + threadIdx.x;
        const bool in = i < e;
        const int64_t s = in ? i : b;
        use[j] = in && bound[s];
        f[j][0] = m[s];
        f[j][1] = red_wants(PART, 1) ? x[s] : 0.0;
        f[j][2] = red_wants(PART, 2) ? y[s] : 0.0;
        f[j][3] = red_wants(PART, 3) ? z[s] : 0.0;
        f[j][4] = red_wants(PART, 4) ? vx[s] : 0.0;
        f[j][5] = red_wants(PART, 5) ? vy[s] : 0.0;
        f[j][6] = red_wants(PART, 6) ? vz[s] : 0.0;
    }
#pragma unroll
    for (int j = 0; j < kSegPer; ++j) {
        if (!use[j]) continue;
        const double mi = f[j][0];
        v[0] += mi;
#pragma unroll
        for (int k = 1; k < 7; ++k)
            if (red_wants(PART, k)) v[k] += mi * f[j][k];
        ++count;
    }
#pragma unroll
    for (int k = 0; k < kRedSums - 1; ++k) sh[k][threadIdx.x] = v[k];
    __shared__ int wcount[kSegThreads / 32];
    int wc = count;
    for (int o = 16; o > 0; o >>= 1) wc += __shfl_down_sync(0xffffffffu, wc, o);
    if ((threadIdx.x & 31) == 0) wcount[threadIdx.x >> 5] = wc;
    __syncthreads();
    if (threadIdx.x < 4 * (kRedSums - 1)) {
        const int k = threadIdx.x % (kRedSums - 1), run = threadIdx.x / (kRedSums - 1);
        double t = 0.0;
        for (int u = run * (kSegThreads / 4); u < (run + 1) * (kSegThreads / 4); ++u) t += sh[k][u];
        q4[k][run] = t;
    }
    __syncthreads();
    if (threadIdx.x < kRedSums - 1) {
        const int k = threadIdx.x;
        if (red_wants(PART, k)) part[(int64_t)c * kRedSums + k] = ((q4[k][0] + q4[k][1]) + q4[k][2]) + q4[k][3];
    } else if (threadIdx.x == kRedSums - 1 && red_wants(PART, 7)) {
        int tot = 0;
        for (int w = 0; w < kSegThreads / 32; ++w) tot += wcount[w];
        part[(int64_t)c * kRedSums + kRedSums - 1] = (double)tot;
    }
}

// One warp per halo: chunk sums added in a fixed order (lane-strided, then the warp tree);
// sets the bound mass, centre of mass, bulk velocity and bound count.
__global__ void ub_reduce_fin_kernel(int nh, const int *__restrict__ cstart, const double *__restrict__ part,
                                     int force, HaloState *hs) {
    const int h = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (h >= nh) return;
    if (!force && !hs[h].active) return;
    double v[kRedSums] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = cstart[h] + lane; c < cstart[h + 1]; c += 32)
#pragma unroll
        for (int k = 0; k < kRedSums; ++k) v[k] += part[(int64_t)c * kRedSums + k];
#pragma unroll
    for (int k = 0; k < kRedSums; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0) {
        HaloState &s = hs[h];
        const double M = v[0];
        s.M = M;
        s.nb = (int)v[7];
        s.sx = v[1]; s.sy = v[2]; s.sz = v[3];
        s.px = v[4]; s.py = v[5]; s.pz = v[6];
        if (M > 0) {
            s.cx = v[1] / M; s.cy = v[2] / M; s.cz = v[3] / M;
            s.vx = v[4] / M; s.vy = v[5] / M; s.vz = v[6] / M;
        } else {
            s.cx = s.cy = s.cz = s.vx = s.vy = s.vz = 0.0;
        }
        if (!force) {   // before the first pass: the reference velocity of the packed velocities
            s.v0x = s.vx; s.v0y = s.vy; s.v0z = s.vz;
            s.wx = s.wy = s.wz = 0.f;
        }
    }
}

// First packing, per member chunk: every member is bound before the first pass, so member
// i of halo h goes to slot i - off[h] of the halo's padded range, re-centred on the halo's
// centre of mass; the chunk holding the halo's end also writes the padding (zero-mass far
// points up to the next multiple of 32).  pk == nullptr writes the velocities alone, pv ==
// nullptr the positions and indices alone.
template <class V>
__global__ void __launch_bounds__(kSegThreads) ub_pack_kernel(
    const int64_t *__restrict__ off, const int64_t *__restrict__ poff, const int *__restrict__ cstart,
    const int *__restrict__ chunk_h, const double *__restrict__ x, const double *__restrict__ y,
    const double *__restrict__ z, const double *__restrict__ m, const double *__restrict__ vx,
    const double *__restrict__ vy, const double *__restrict__ vz, const HaloState *__restrict__ hs,
    V *__restrict__ pk, float4 *__restrict__ pv, int *__restrict__ pidx) {
    const int c = blockIdx.x;
    const int h = chunk_h[c];
    const double cx = hs[h].cx, cy = hs[h].cy, cz = hs[h].cz;
    const double v0x = hs[h].v0x, v0y = hs[h].v0y, v0z = hs[h].v0z;
    const int64_t hb = off[h], he = off[h + 1], pb = poff[h];
    const int64_t b = hb + (int64_t)(c - cstart[h]) * kSeg;
    const int64_t e = min(he, b + kSeg);
    for (int64_t i = b + threadIdx.x; i < e; i += kSegThreads) {
        if (pk) {
            V r;
            r.x = x[i] - cx; r.y = y[i] - cy; r.z = z[i] - cz; r.w = m[i];
            pk[pb + (i - hb)] = r;
            pidx[pb + (i - hb)] = (int)i;
        }
        // FP32 path: velocity relative to the bulk velocity at packing, and the mass
        if (pv) pv[pb + (i - hb)] = make_float4((float)(vx[i] - v0x), (float)(vy[i] - v0y), (float)(vz[i] - v0z),
                                                 (float)m[i]);
    }
    if (e == he) {
        const int64_t nb = he - hb, npad = (nb + 31) & ~31ll;
        for (int64_t r = nb + threadIdx.x; r < npad; r += kSegThreads) {
            if (pk) {
                V f;
                f.x = f.y = f.z = kFar; f.w = 0;
                pk[pb + r] = f;
                pidx[pb + r] = -1;
            }
            if (pv) pv[pb + r] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// Work list for the pair kernel: haloes in decreasing initial size, tiles of 32*T targets.
// Also records the pass's pair count (sum of nb^2 over active haloes) in pairs_out.
__device__ __forceinline__ int tile_t_for(const TileTable &tab, int nb) {
    for (int c = 0; c < tab.n; ++c)
        if (nb <= tab.upper[c]) return tab.t[c];
    return 4;
}

// The work list is implicit: ordered halo q owns items istart[q] .. istart[q+1]-1, described
// by idesc[q] = (halo, T, slices, unused); item i of that halo is (tile i / slices,
// slice i % slices).  Only nh+1 prefix counts are written per pass.
// The same pass also lays out the energy segments: active ordered halo q owns segments
// sstart[q] .. sstart[q+1]-1 of kSeg slots each; sown[seg] names the segment's ordered halo.

__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Full passes over a halo of more than kSymBlock bound particles use the symmetric block
// kernel instead: blocks of kSymBlock slots, one item per block pair (tb <= sb), B(B+1)/2
// items for B blocks, listed from ystart[q]; the partial sums are then kept per block
// (B slices of kSymBlock).  idesc[q].w is the number of partial slices the energy kernel adds.
constexpr int kSymWarps = 4, kSymT = 8;
constexpr int kSymBlock = kSymWarps * 32 * kSymT;   // 1024 slots

// The pass's work list, built in three steps over the haloes in size order (q):
//   count - per halo q: its halo h, tile shape, source slices, and three counts: warp items
//           (tiles x slices), energy segments, symmetric block-pair items (0 unless active);
//   scan  - exclusive prefix sums of the three counts (CUB);
//   fill  - the prefix sums become istart / sstart / ystart, every segment records its owner
//           (sown), and the totals go to cnt[] (warp items, energy segments, block-pair items,
//           their counters reset) and to the last entries of the start arrays.
// With pairs_out (profiling), the pass's pair terms (nb x sources, all haloes) and those of the
// haloes on the symmetric block kernel are summed into pairs_out[0..1] (zeroed beforehand).
__global__ void __launch_bounds__(256) ub_items_count_kernel(int nh, const int *__restrict__ order,
                                                             const HaloState *hs, TileTable tab, int slice_len,
                                                             int inc, int sym_ok, int4 *__restrict__ counts,
                                                             int4 *__restrict__ idesc,
                                                             unsigned long long *__restrict__ pairs_out) {
    const int lane = threadIdx.x & 31;
    for (int q0 = blockIdx.x * blockDim.x; q0 < nh; q0 += gridDim.x * blockDim.x) {
        const int q = q0 + threadIdx.x;
        int h = -1, n = 0, T = 4, nsl = 1, nseg = 0, ny = 0, nsl_e = 0;
        unsigned long long my_pairs = 0, my_spairs = 0;
        if (q < nh) {
            h = order[q];
            if (hs[h].active) {
                const int nb = hs[h].nb;
                const int ns = inc ? hs[h].nrem : nb;   // sources: removed particles or the halo itself
                T = tile_t_for(tab, nb);
                nsl = (int)(((int64_t)ns + slice_len - 1) / slice_len);
                if (!inc && sym_ok && nb > kSymBlock && nb <= 65535 * kSymBlock) {
                    const int B = (nb + kSymBlock - 1) / kSymBlock;   // B <= 65535: B(B+1)/2 < 2^31
                    ny = (int)((int64_t)B * (B + 1) / 2);
                    nsl_e = B;
                    my_spairs = (unsigned long long)nb * (unsigned long long)nb;
                } else {
                    n = ns > 0 ? ((nb + 32 * T - 1) / (32 * T)) * nsl : 0;
                    nsl_e = nsl;
                }
                nseg = max(1, (nb + kSeg - 1) / kSeg);
                my_pairs = (unsigned long long)nb * (unsigned long long)ns;
            }
            counts[q] = make_int4(n, nseg, ny, 0);
            idesc[q] = make_int4(h, T, max(nsl, 1), nsl_e);
        }
        if (pairs_out) {   // one atomic per warp
            for (int o = 16; o > 0; o >>= 1) {
                my_pairs += __shfl_xor_sync(0xffffffffu, my_pairs, o);
                my_spairs += __shfl_xor_sync(0xffffffffu, my_spairs, o);
            }
            if (lane == 0 && (my_pairs | my_spairs)) {
                atomicAdd(pairs_out, my_pairs);
                atomicAdd(pairs_out + 1, my_spairs);
            }
        }
    }
}

__global__ void __launch_bounds__(256) ub_items_fill_kernel(int nh, const int4 *__restrict__ counts,
                                                            const int4 *__restrict__ pre, int *__restrict__ istart,
                                                            int *__restrict__ ystart, int *__restrict__ sstart,
                                                            int *__restrict__ sown, int *__restrict__ cnt) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nh; q += gridDim.x * blockDim.x) {
        const int4 c = counts[q], p = pre[q];
        istart[q] = p.x;
        sstart[q] = p.y;
        ystart[q] = p.z;
        for (int sg = 0; sg < c.y; ++sg) sown[p.y + sg] = q;
        if (q == nh - 1) {
            istart[nh] = p.x + c.x;
            sstart[nh] = p.y + c.y;
            ystart[nh] = p.z + c.z;
            cnt[0] = p.x + c.x;   // warp items
            cnt[1] = 0;           // their counter
            cnt[2] = p.y + c.y;   // energy segments
            cnt[3] = p.z + c.z;   // symmetric block items
            cnt[4] = 0;           // their counter
        }
    }
}

// 32 sources of the staged chunk against T targets, two sources per f32x2 instruction.
// sa[kp] = {x_2kp, x_2kp+1, y_2kp, y_2kp+1}, sb[kp] = {z.., z.., m.., m..}.  Each target keeps
// an {even, odd} pair of partial sums.  SELF: target ts skips the source in its own lane slot.
template <int T, bool SELF>
__device__ __forceinline__ void chunk_pairs(const float4 *sa, const float4 *sb, const f2x (&tx)[T], const f2x (&ty)[T],
                                            const f2x (&tz)[T], f2x e2, f2x (&acc)[T], int ts, int lane) {
#pragma unroll 4
    for (int kp = 0; kp < 16; ++kp) {
        const float4 a = sa[kp], b = sb[kp];
        const f2x X = pack2(a.x, a.y), Y = pack2(a.z, a.w), Z = pack2(b.x, b.y), M = pack2(b.z, b.w);
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const f2x dx = sub2(X, tx[t]), dy = sub2(Y, ty[t]), dz = sub2(Z, tz[t]);
            f2x r2 = fma2(dz, dz, e2);
            r2 = fma2(dy, dy, r2);
            r2 = fma2(dx, dx, r2);
            float r0, r1;
            unpack2(r2, r0, r1);
            float i0 = rsqrt_ftz(r0), i1 = rsqrt_ftz(r1);
            if (SELF && t == ts && kp == (lane >> 1)) {
                if (lane & 1) i1 = 0.f;
                else i0 = 0.f;
            }
            acc[t] = fma2(M, pack2(i0, i1), acc[t]);
        }
    }
}

// One work item: 32*T target slots of one halo (tpk) against source chunks [c_begin, c_end)
// of spk.  self_ok: targets and sources are the same slots, so the self pair is skipped.
template <int T>
__device__ __forceinline__ void pair_item(const float4 *__restrict__ tpk, const float4 *__restrict__ pk, int64_t base,
                                          int nb, int tile, float eps2, int c_begin, int c_end, bool self_ok,
                                          float2 *__restrict__ out, float4 *buf, int lane) {
    {
        f2x tx[T], ty[T], tz[T];
        float sum[T], comp[T];
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const int r = tile * 32 * T + t * 32 + lane;
            const float4 p = r < nb ? tpk[base + r] : make_float4(kFar, kFar, kFar, 0.f);
            tx[t] = pack2(p.x, p.x);
            ty[t] = pack2(p.y, p.y);
            tz[t] = pack2(p.z, p.z);
            sum[t] = 0.f;
            comp[t] = 0.f;
        }
        const f2x e2 = pack2(eps2, eps2);
        float *sa = reinterpret_cast<float *>(buf);        // 16 float4: x/y pairs
        float *sb = reinterpret_cast<float *>(buf + 16);   // 16 float4: z/m pairs
        const int kp = lane >> 1, hf = lane & 1;
        const int self0 = tile * T;   // chunk c holds the self slot of target t = c - self0
        float4 nxt = pk[base + (int64_t)c_begin * 32 + lane];
        for (int c = c_begin; c < c_end; ++c) {
            __syncwarp();
            sa[kp * 4 + hf] = nxt.x;
            sa[kp * 4 + 2 + hf] = nxt.y;
            sb[kp * 4 + hf] = nxt.z;
            sb[kp * 4 + 2 + hf] = nxt.w;
            __syncwarp();
            if (c + 1 < c_end) nxt = pk[base + (int64_t)(c + 1) * 32 + lane];
            f2x acc[T];
#pragma unroll
            for (int t = 0; t < T; ++t) acc[t] = pack2(0.f, 0.f);
            const int ts = c - self0;
            if (self_ok && ts >= 0 && ts < T)
                chunk_pairs<T, true>(buf, buf + 16, tx, ty, tz, e2, acc, ts, lane);
            else
                chunk_pairs<T, false>(buf, buf + 16, tx, ty, tz, e2, acc, ts, lane);
#pragma unroll
            for (int t = 0; t < T; ++t) {
                float a0, a1;
                unpack2(acc[t], a0, a1);
                two_sum_acc(sum[t], comp[t], a0 + a1);
            }
        }
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const int r = tile * 32 * T + t * 32 + lane;
            if (r < nb) out[r] = df_from_acc(sum[t], comp[t]);
        }
    }
}

// Persistent all-pairs kernel over the work list (FP32 pair terms, compensated sums).  An
// item is (halo, target tile, tile shape T, source slice): 32*T targets against one slice of
// slice_chunks*32 source slots.  Each slice writes its own partial sums
// (part[qoff[h] + slice * npad_h + r]); the energy kernel adds the slices in order, so the
// result does not depend on which warp ran which item.  Full passes take the sources from the
// targets' own slots (self pair skipped); incremental passes (inc) take them from the slots of
// the particles removed by the previous pass (spk, hs.nrem of them), whose contribution the
// energy kernel then subtracts from the previous potential.
__global__ void __launch_bounds__(256) ub_pair_kernel(const float4 *__restrict__ pk, const float4 *__restrict__ spk,
                                                      int inc, const int64_t *__restrict__ poff,
                                                      const int64_t *__restrict__ qoff, const HaloState *__restrict__ hs,
                                                      int nh, const int *__restrict__ istart,
                                                      const int4 *__restrict__ idesc, const int *__restrict__ nitems_p,
                                                      int *counter, float eps2, int slice_chunks,
                                                      float2 *__restrict__ part) {
    __shared__ float4 buf[kUbWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nitems = *nitems_p;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(counter, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nitems) break;
        // ordered halo owning the item: last q with istart[q] <= item
        int lo = 0, hi = nh - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (istart[mid] <= item) lo = mid;
            else hi = mid - 1;
        }
        const int4 d = idesc[lo];
        const int local = item - istart[lo];
        const int4 it = make_int4(d.x, local / d.z, d.y, local % d.z);
        const int h = it.x, tile = it.y, slice = it.w;
        const int64_t base = poff[h];
        const int64_t npad = poff[h + 1] - base;
        const int nb = hs[h].nb;
        const int ns = inc ? hs[h].nrem : nb;
        const float4 *src = inc ? spk : pk;
        const int c0 = slice * slice_chunks;
        const int c1 = min((ns + 31) >> 5, c0 + slice_chunks);
        float2 *out = part + qoff[h] + (int64_t)slice * npad;
        switch (it.z) {
            case 1: pair_item<1>(pk, src, base, nb, tile, eps2, c0, c1, !inc, out, buf[w], lane); break;
            case 2: pair_item<2>(pk, src, base, nb, tile, eps2, c0, c1, !inc, out, buf[w], lane); break;
            default: pair_item<4>(pk, src, base, nb, tile, eps2, c0, c1, !inc, out, buf[w], lane); break;
        }
    }
}

// Reduce-scatter of 16 per-lane values across the warp: lanes l and l^1 end with the warp's
// total of value (l >> 1) & 15 (fixed association: halving steps over lane bits 4..1, then
// the pair l, l^1).
__device__ __forceinline__ float warp_reduce_scatter16(float (&v)[16], int lane) {
    float a[8], b[4], c[2];
    {
        const bool up = lane & 16;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float send = up ? v[k] : v[k + 8], keep = up ? v[k + 8] : v[k];
            a[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
        }
    }
    {
        const bool up = lane & 8;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float send = up ? a[k] : a[k + 4], keep = up ? a[k + 4] : a[k];
            b[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
        }
    }
    {
        const bool up = lane & 4;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const float send = up ? b[k] : b[k + 2], keep = up ? b[k + 2] : b[k];
            c[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
        }
    }
    const bool up = lane & 2;
    const float send = up ? c[0] : c[1], keep = up ? c[1] : c[0];
    const float d = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    return d + __shfl_xor_sync(0xffffffffu, d, 1);
}

// Symmetric form of chunk_pairs: every pair term 1/r is used twice, m_source / r for the
// lane's targets (acc, as in chunk_pairs) and m_target / r for the chunk's sources.  The
// source side is summed over the lane's T targets, then over the warp (reduce-scatter), and
// the warp's 32 * T-target sums of the chunk's 32 sources go to sout[0..32).
template <int T>
__device__ __forceinline__ void chunk_pairs_sym(const float4 *sa, const float4 *sb, const f2x (&tx)[T],
                                                const f2x (&ty)[T], const f2x (&tz)[T], const f2x (&tm)[T], f2x e2,
                                                f2x (&acc)[T], float *sout, int lane) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        f2x sacc[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) sacc[k] = pack2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float4 a = sa[half * 8 + k], b = sb[half * 8 + k];
            const f2x X = pack2(a.x, a.y), Y = pack2(a.z, a.w), Z = pack2(b.x, b.y), M = pack2(b.z, b.w);
#pragma unroll
            for (int t = 0; t < T; ++t) {
                const f2x dx = sub2(X, tx[t]), dy = sub2(Y, ty[t]), dz = sub2(Z, tz[t]);
                f2x r2 = fma2(dz, dz, e2);
                r2 = fma2(dy, dy, r2);
                r2 = fma2(dx, dx, r2);
                float r0, r1;
                unpack2(r2, r0, r1);
                const f2x ri = pack2(rsqrt_ftz(r0), rsqrt_ftz(r1));
                acc[t] = fma2(M, ri, acc[t]);
                sacc[k] = fma2(tm[t], ri, sacc[k]);
            }
        }
        float v[16];
#pragma unroll
        for (int k = 0; k < 8; ++k) unpack2(sacc[k], v[2 * k], v[2 * k + 1]);
        const float s = warp_reduce_scatter16(v, lane);
        if ((lane & 1) == 0) sout[half * 16 + (lane >> 1)] = s;
    }
}

// Full passes over the haloes of more than kSymBlock bound particles.  The halo's slots are
// cut into blocks of kSymBlock; an item is a block pair (tb, sb), tb <= sb, taken by one CTA
// from an atomic counter.  The CTA (4 warps of 8 targets per lane, so that the source-side
// reduce-scatter serves 8 targets) stages the source block in shared memory; warp w holds
// targets tb*kSymBlock + w*256 + t*32 + lane.  Diagonal items (tb == sb) are plain (self pair
// skipped) and write the targets' partial for slice sb.  Off-diagonal items compute each pair
// once: the targets' partial goes to slice sb (part[qoff + sb*npad + r]) and the sources'
// partial -- per source, the 4 warps' sums added in warp order, compensated -- to slice tb.  So
// slot r of block b receives slice k from item (b, k) for k >= b and from item (k, b) for
// k < b: every slice exactly once, and the energy kernel adds slices 0..B-1 in order.
__global__ void __launch_bounds__(128) ub_pair_sym_kernel(const float4 *__restrict__ pk,
                                                          const int64_t *__restrict__ poff,
                                                          const int64_t *__restrict__ qoff,
                                                          const HaloState *__restrict__ hs, int nh,
                                                          const int *__restrict__ ystart,
                                                          const int4 *__restrict__ idesc, const int *__restrict__ cnt,
                                                          int *counter, float eps2, float2 *__restrict__ part) {
    extern __shared__ float4 sym_smem[];
    float4 *ssrc = sym_smem;                                            // 32 chunks x (16 + 16) float4
    float *spart = reinterpret_cast<float *>(sym_smem + kSymBlock);     // [kSymWarps][kSymBlock]
    __shared__ int4 job;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nitems = cnt[3];
    const f2x e2 = pack2(eps2, eps2);
    for (;;) {
        if (threadIdx.x == 0) {
            const int item = atomicAdd(counter, 1);
            int4 jb = make_int4(-1, 0, 0, 0);
            if (item < nitems) {
                int lo = 0, hi = nh - 1;   // ordered halo owning the item: last q with ystart[q] <= item
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (ystart[mid] <= item) lo = mid;
                    else hi = mid - 1;
                }
                const int h = idesc[lo].x;
                const int64_t u = item - ystart[lo];
                const int64_t B = (hs[h].nb + kSymBlock - 1) / kSymBlock;
                // row tb of the upper triangle starts at tb*B - tb*(tb-1)/2
                int64_t tb = (int64_t)(((double)(2 * B + 1) - sqrt((double)(2 * B + 1) * (double)(2 * B + 1) -
                                                                     8.0 * (double)u)) * 0.5);
                tb = tb < 0 ? 0 : (tb > B - 1 ? B - 1 : tb);
                while (tb + 1 < B && (tb + 1) * B - (tb + 1) * tb / 2 <= u) ++tb;
                while (tb > 0 && tb * B - tb * (tb - 1) / 2 > u) --tb;
                const int64_t sb = tb + (u - (tb * B - tb * (tb - 1) / 2));
                jb = make_int4(h, (int)tb, (int)sb, 0);
            }
            job = jb;
        }
        __syncthreads();
        const int4 jb = job;
        if (jb.x < 0) break;
        const int h = jb.x, tb = jb.y, sb = jb.z;
        const bool sym = tb != sb;
        const int64_t base = poff[h], npad = poff[h + 1] - base;
        const int nb = hs[h].nb;
        const int s0 = sb * kSymBlock;
        const int nch = min(kSymBlock / 32, (nb - s0 + 31) >> 5);   // chunks holding sources
        // stage the source block (slots past nb: zero mass, far away)
        for (int k = threadIdx.x; k < nch * 32; k += blockDim.x) {
            const int s = s0 + k;
            const float4 p = s < nb ? pk[base + s] : make_float4(kFar, kFar, kFar, 0.f);
            float *ca = reinterpret_cast<float *>(ssrc + (k >> 5) * 32);
            const int li = k & 31, kp = li >> 1, hf = li & 1;
            ca[kp * 4 + hf] = p.x;
            ca[kp * 4 + 2 + hf] = p.y;
            ca[64 + kp * 4 + hf] = p.z;
            ca[64 + kp * 4 + 2 + hf] = p.w;
        }
        __syncthreads();
        const int t0 = tb * kSymBlock + w * 32 * kSymT;   // the warp's first target slot
        float *sp = spart + w * kSymBlock;
        if (t0 < nb) {
            f2x tx[kSymT], ty[kSymT], tz[kSymT], tm[kSymT];
            float sum[kSymT], comp[kSymT];
#pragma unroll
            for (int t = 0; t < kSymT; ++t) {
                const int r = t0 + t * 32 + lane;
                const float4 p = r < nb ? pk[base + r] : make_float4(kFar, kFar, kFar, 0.f);
                tx[t] = pack2(p.x, p.x);
                ty[t] = pack2(p.y, p.y);
                tz[t] = pack2(p.z, p.z);
                tm[t] = pack2(p.w, p.w);
                sum[t] = 0.f;
                comp[t] = 0.f;
            }
            for (int c = 0; c < nch; ++c) {
                const float4 *ca = ssrc + c * 32;
                f2x acc[kSymT];
#pragma unroll
                for (int t = 0; t < kSymT; ++t) acc[t] = pack2(0.f, 0.f);
                if (sym) {
                    chunk_pairs_sym<kSymT>(ca, ca + 16, tx, ty, tz, tm, e2, acc, sp + c * 32, lane);
                } else {
                    const int ts = c - w * kSymT;   // chunk c holds the self slot of target ts
                    if (ts >= 0 && ts < kSymT)
                        chunk_pairs<kSymT, true>(ca, ca + 16, tx, ty, tz, e2, acc, ts, lane);
                    else
                        chunk_pairs<kSymT, false>(ca, ca + 16, tx, ty, tz, e2, acc, ts, lane);
                }
#pragma unroll
                for (int t = 0; t < kSymT; ++t) {
                    float a0, a1;
                    unpack2(acc[t], a0, a1);
                    two_sum_acc(sum[t], comp[t], a0 + a1);
                }
            }
            float2 *out = part + qoff[h] + (int64_t)sb * npad;
#pragma unroll
            for (int t = 0; t < kSymT; ++t) {
                const int r = t0 + t * 32 + lane;
                if (r < nb) out[r] = df_from_acc(sum[t], comp[t]);
            }
        } else if (sym) {
            for (int k = lane; k < nch * 32; k += 32) sp[k] = 0.f;   // no targets here: no terms
        }
        if (sym) {
            __syncthreads();
            float2 *out = part + qoff[h] + (int64_t)tb * npad;
            for (int k = threadIdx.x; k < nch * 32; k += blockDim.x) {
                const int s = s0 + k;
                if (s < nb) {
                    float sum = 0.f, comp = 0.f;   // the warps' sums in warp order, compensated
#pragma unroll
                    for (int ww = 0; ww < kSymWarps; ++ww) two_sum_acc(sum, comp, spart[ww * kSymBlock + k]);
                    out[s] = df_from_acc(sum, comp);
                }
            }
        }
        __syncthreads();   // shared memory is restaged by the next item
    }
}

// The end of a pass runs in three kernels:
//   energy  - per energy segment (kSeg packed slots of one halo, so a big halo is spread over
//             many blocks): FP64 energy and sign test of every slot; removed particles are
//             marked; per-segment FP64 sums of the survivors (count, mass, mass-weighted
//             velocity) and of the pass's kinetic / potential energy.  The centre of mass is
//             not needed between passes (positions stay re-centred on the first pass's
//             centre) and is recomputed over the final bound set after the last pass;
//   finalize- one warp per halo: segment sums added in a fixed order (deterministic):
//             removals, pass count, energies, the next pass's mass and bulk velocity, and the
//             survivors / removed particles before each segment.  A halo whose pass removed
//             nothing becomes inactive;
//   compact - per segment of a halo still active: survivors copied, in order, into the other
//             packed buffer, removed particles into the next pass's source list.
constexpr int kSegSums = 8;   // removed, kept, ekin, epot, M, Mvx, Mvy, Mvz

template <class V>
__global__ void __launch_bounds__(kSegThreads) ub_energy_seg_kernel(
    const int *__restrict__ sstart, const int *__restrict__ sown, const int4 *__restrict__ idesc,
    const int *__restrict__ nsegs, const int64_t *__restrict__ poff, const int64_t *__restrict__ qoff,
    int inc, const int *__restrict__ pidx, const double *__restrict__ part,
    const double *__restrict__ phi_prev, double *__restrict__ phi_cur, const double *__restrict__ vx,
    const double *__restrict__ vy, const double *__restrict__ vz, const double *__restrict__ m, double gfac,
    const HaloState *__restrict__ hs, unsigned char *__restrict__ bound, double *__restrict__ phi_out,
    unsigned char *__restrict__ keepf, double *__restrict__ seg_sums) {
    const int seg = blockIdx.x;
    if (seg >= *nsegs) return;
    __shared__ double sh[kSegSums][32];
    const int q = sown[seg];
    const int h = idesc[q].x;
    const int sl = seg - sstart[q];
    const HaloState s = hs[h];
    const int64_t pb = poff[h], npad = poff[h + 1] - pb, qb = qoff[h];
    const int nsl = idesc[q].w;   // partial-sum slices written by this pass's pair kernels
    const int rend = min(s.nb, (sl + 1) * kSeg);
    // the segment's kSegPer slots per thread are loaded together (independent gathers in
    // flight), then evaluated in slot order
    int r[kSegPer], ii[kSegPer];
    double d[kSegPer];
#pragma unroll
    for (int j = 0; j < kSegPer; ++j) {
        r[j] = sl * kSeg + j * kSegThreads + threadIdx.x;
        ii[j] = r[j] < rend ? pidx[pb + r[j]] : -1;
        d[j] = 0.0;
    }
    for (int k = 0; k < nsl; ++k)   // slices in order
#pragma unroll
        for (int j = 0; j < kSegPer; ++j)
            if (ii[j] >= 0) d[j] += part[qb + (int64_t)k * npad + r[j]];
    // gathers of all the thread's slots issued together (predicated, no branch between them)
    double gv[kSegPer][4], pprev[kSegPer];
#pragma unroll
    for (int j = 0; j < kSegPer; ++j) {
        const int i = ii[j];
        const bool ok = i >= 0;
        gv[j][0] = ok ? vx[i] : 0.0;
        gv[j][1] = ok ? vy[i] : 0.0;
        gv[j][2] = ok ? vz[i] : 0.0;
        gv[j][3] = ok ? m[i] : 0.0;
        pprev[j] = (ok && inc) ? phi_prev[pb + r[j]] : 0.0;
    }
    double v[kSegSums] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int j = 0; j < kSegPer; ++j) {
        const int i = ii[j];
        if (i < 0) continue;
        const double dvx = gv[j][0] - s.vx, dvy = gv[j][1] - s.vy, dvz = gv[j][2] - s.vz;
        const double ek = 0.5 * (dvx * dvx + dvy * dvy + dvz * dvz);
        // full pass: the sum itself; incremental pass: previous potential minus the removed
        // particles' contribution
        const double p = inc ? pprev[j] - d[j] : d[j];
        phi_cur[pb + r[j]] = p;
        const double e = ek - gfac * p;
        const bool keep = !(e > 0.0);
        keepf[pb + r[j]] = keep ? 1 : 0;
        if (!keep) {
            bound[i] = 0;
            v[0] += 1.0;
            if (phi_out) phi_out[i] = 0.0;
        } else {
            const double mi = gv[j][3];
            v[1] += 1.0;
            v[2] += mi * ek;
            v[3] += mi * p;
            v[4] += mi;
            v[5] += mi * gv[j][0];
            v[6] += mi * gv[j][1];
            v[7] += mi * gv[j][2];
            if (phi_out) phi_out[i] = p;
        }
    }
    block_sum_store<kSegSums>(v, sh, seg_sums + (int64_t)seg * kSegSums);
}

// One warp per active ordered halo, after the energy pass: the halo's segment sums added in a
// fixed order (lane-strided, then the warp tree), so the result does not depend on timing;
// removals, pass count, energies and the next pass's mass, centre and bulk velocity.  A halo
// whose pass removed nothing becomes inactive.  Also writes, per segment, the survivors and
// removed particles of the halo's earlier segments (seg_pre), where compaction starts writing.
__global__ void ub_finalize_kernel(int nh, const int *__restrict__ order, const int *__restrict__ sstart,
                                   const double *__restrict__ seg_sums, double gfac, HaloState *hs,
                                   int2 *__restrict__ seg_pre) {
    const int q = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (q >= nh) return;
    const int h = order[q];
    if (!hs[h].active) return;
    const int s0 = sstart[q], s1 = sstart[q + 1];
    double v[kSegSums] = {0, 0, 0, 0, 0, 0, 0, 0};
    int keep_run = 0, rem_run = 0;
    for (int b0 = s0; b0 < s1; b0 += 32) {
        const int sg = b0 + lane;
        const bool ok = sg < s1;
        const int nrem = ok ? (int)seg_sums[(int64_t)sg * kSegSums + 0] : 0;
        const int nkeep = ok ? (int)seg_sums[(int64_t)sg * kSegSums + 1] : 0;
        const int ri = warp_incl_scan(nrem, lane), ki = warp_incl_scan(nkeep, lane);
        if (ok) seg_pre[sg] = make_int2(keep_run + ki - nkeep, rem_run + ri - nrem);
        keep_run += __shfl_sync(0xffffffffu, ki, 31);
        rem_run += __shfl_sync(0xffffffffu, ri, 31);
        if (ok)
#pragma unroll
            for (int k = 0; k < kSegSums; ++k) v[k] += seg_sums[(int64_t)sg * kSegSums + k];
    }
#pragma unroll
    for (int k = 0; k < kSegSums; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0) {
        HaloState &o = hs[h];
        o.nprev = o.nb;
        o.removed = (int)v[0];
        o.nrem = (int)v[0];
        o.iter += 1;
        o.ekin = v[2];
        o.epot = -0.5 * gfac * v[3];
        if (v[0] == 0.0) {
            o.active = 0;
        } else {
            const double M = v[4];
            o.M = M;
            o.nb = (int)v[1];
            if (M > 0) {
                o.vx = v[5] / M; o.vy = v[6] / M; o.vz = v[7] / M;
            } else {
                o.vx = o.vy = o.vz = 0.0;
            }
        }
    }
}

// Per segment of a halo that stays active: survivors copied in order into the other packed
// buffer (with their potential, the next incremental pass's starting point), removed
// particles into the removed list (the next pass's sources); the halo's last segment pads
// both to a multiple of 32 with zero-mass far points.
template <class V>
__global__ void __launch_bounds__(kSegThreads) ub_compact_seg_kernel(
    const int *__restrict__ sstart, const int *__restrict__ sown, const int4 *__restrict__ idesc,
    const int *__restrict__ nsegs, const int64_t *__restrict__ poff, const HaloState *__restrict__ hs,
    const unsigned char *__restrict__ keepf, const int2 *__restrict__ seg_pre, const V *__restrict__ pk_in,
    const int *__restrict__ pidx_in, const double *__restrict__ phi_cur, V *__restrict__ pk_out,
    int *__restrict__ pidx_out, double *__restrict__ phi_next, V *__restrict__ removed) {
    const int seg = blockIdx.x;
    if (seg >= *nsegs) return;
    __shared__ int wcount[kSegThreads / 32], wrem[kSegThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int q = sown[seg];
    const int h = idesc[q].x;
    if (!hs[h].active) return;   // converged this pass: its packed slots are not read again
    const int s0 = sstart[q], sl = seg - s0, nseg = sstart[q + 1] - s0;
    const int nb = hs[h].nprev;
    const int64_t pb = poff[h];
    const int2 pre = seg_pre[seg];
    int running = pre.x, rrunning = pre.y;
    const int rend = min(nb, (sl + 1) * kSeg);
    for (int r0 = sl * kSeg; r0 < rend; r0 += kSegThreads) {
        const int r = r0 + threadIdx.x;
        const bool valid = r < rend;
        const bool keep = valid && keepf[pb + r];
        const bool gone = valid && !keep;
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        const unsigned bgone = __ballot_sync(0xffffffffu, gone);
        if (lane == 0) {
            wcount[w] = __popc(bal);
            wrem[w] = __popc(bgone);
        }
        __syncthreads();
        int rank = running, rrank = rrunning, tot = 0, trem = 0;
#pragma unroll
        for (int k = 0; k < kSegThreads / 32; ++k) {
            if (k < w) {
                rank += wcount[k];
                rrank += wrem[k];
            }
            tot += wcount[k];
            trem += wrem[k];
        }
        rank += __popc(bal & ((1u << lane) - 1u));
        rrank += __popc(bgone & ((1u << lane) - 1u));
        if (keep) {
            pk_out[pb + rank] = pk_in[pb + r];
            pidx_out[pb + rank] = pidx_in[pb + r];
            phi_next[pb + rank] = phi_cur[pb + r];
        } else if (gone) {
            removed[pb + rrank] = pk_in[pb + r];
        }
        running += tot;
        rrunning += trem;
        __syncthreads();
    }
    if (sl == nseg - 1) {   // the halo's last segment pads after the survivors and the removed
        V f;
        f.x = f.y = f.z = kFar;
        f.w = 0;
        const int nkeep = running, nrem = rrunning;
        for (int r = nkeep + threadIdx.x; r < ((nkeep + 31) & ~31); r += kSegThreads) {
            pk_out[pb + r] = f;
            pidx_out[pb + r] = -1;
        }
        for (int r = nrem + threadIdx.x; r < ((nrem + 31) & ~31); r += kSegThreads) removed[pb + r] = f;
    }
}

// ---- end of a pass, FP32 path: per-particle work in FP32 and double-float only ----
// This GPU's FP64 rate is a small fraction of its FP32 rate, so the per-particle work of the
// FP32 path runs without FP64: the potential is a double-float (about 48 bits) carried from
// pass to pass, the energy and its sign test are FP32 (relative error ~1e-7, far inside the
// 1e-5 band where FP32 pair sums already leave the cut undecided), and the packed velocities
// are FP32 offsets from the bulk velocity at packing.  The halo's FP64 mass and sums of m x
// and m v are not re-summed over the survivors: each pass subtracts the FP64 sums over the
// particles it removed (gathered from the caller's FP64 arrays), usually a few per cent.
struct SegDF {
    int removed, kept;
    float2 ekin, epot;                            // double-float sums over the survivors: m ek, m phi
    double rm, rmx, rmy, rmz, rmvx, rmvy, rmvz;   // FP64 sums over the removed particles
};

__device__ __forceinline__ float2 df_warp_sum(float2 v) {
    for (int o = 16; o > 0; o >>= 1)
        v = df_add(v, make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o)));
    return v;
}

// Per energy segment: potential phi (double-float: the slices' partials added in order, or,
// in an incremental pass, the previous potential minus them), FP32 energy
// E = 1/2 |u - w|^2 - G factor_v^2 phi with u the packed velocity offset and w the halo's
// current bulk-velocity offset, sign test; survivors' sums of m ek and m phi in double-float;
// the removed particles are listed in slot order and their FP64 mass, m x and m v summed by
// warp 0 from the caller's arrays.
__global__ void __launch_bounds__(kSegThreads) ub_energy_df_kernel(
    const int *__restrict__ sstart, const int *__restrict__ sown, const int4 *__restrict__ idesc,
    const int *__restrict__ nsegs, const int64_t *__restrict__ poff, const int64_t *__restrict__ qoff, int inc,
    const int *__restrict__ pidx, const float4 *__restrict__ pv, const float2 *__restrict__ part,
    const float2 *__restrict__ phi_prev, float2 *__restrict__ phi_cur, const double *__restrict__ x,
    const double *__restrict__ y, const double *__restrict__ z, const double *__restrict__ vx,
    const double *__restrict__ vy, const double *__restrict__ vz, const double *__restrict__ m, float gfac,
    const HaloState *__restrict__ hs, unsigned char *__restrict__ bound, double *__restrict__ phi_out,
    unsigned char *__restrict__ keepf, SegDF *__restrict__ seg_sums) {
    __shared__ unsigned char gone[kSeg];
    __shared__ int rlist[kSeg];
    __shared__ float2 se[2][kSegThreads / 32];
    __shared__ int sc[2][kSegThreads / 32];
    const int nseg_all = *nsegs;
    for (int seg = blockIdx.x; seg < nseg_all; seg += gridDim.x) {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int q = sown[seg];
        const int h = idesc[q].x;
        const int nsl = idesc[q].w;   // partial-sum slices written by this pass's pair kernels
        const int sl = seg - sstart[q];
        const int nb = hs[h].nb;
        const float wx = hs[h].wx, wy = hs[h].wy, wz = hs[h].wz;
        const int64_t pb = poff[h], npad = poff[h + 1] - pb, qb = qoff[h];
        const int rend = min(nb, (sl + 1) * kSeg);
        int r[kSegPer];
        bool ok[kSegPer];
        float4 u[kSegPer];
        float2 d[kSegPer];
#pragma unroll
        for (int j = 0; j < kSegPer; ++j) {
            r[j] = sl * kSeg + j * kSegThreads + threadIdx.x;
            ok[j] = r[j] < rend;
            u[j] = ok[j] ? pv[pb + r[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
            d[j] = make_float2(0.f, 0.f);
        }
        // slices in order, four at a time with all their loads issued before the additions
        const float2 *pr[kSegPer];
#pragma unroll
        for (int j = 0; j < kSegPer; ++j) pr[j] = part + qb + (ok[j] ? r[j] : 0);
        int k = 0;
        for (; k + 4 <= nsl; k += 4) {
            float2 t[4][kSegPer];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                for (int j = 0; j < kSegPer; ++j) t[kk][j] = pr[j][(int64_t)(k + kk) * npad];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                for (int j = 0; j < kSegPer; ++j)
                    if (ok[j]) d[j] = df_add(d[j], t[kk][j]);
        }
        for (; k < nsl; ++k)
#pragma unroll
            for (int j = 0; j < kSegPer; ++j)
                if (ok[j]) d[j] = df_add(d[j], pr[j][(int64_t)k * npad]);
        float ek_s = 0.f, ek_c = 0.f, ep_s = 0.f, ep_c = 0.f;
        int kept = 0, removed = 0;
#pragma unroll
        for (int j = 0; j < kSegPer; ++j) {
            const int slot = j * kSegThreads + threadIdx.x;   // within the segment
            if (!ok[j]) {
                gone[slot] = 0;
                continue;
            }
            // full pass: the sum itself; incremental pass: previous potential minus the removed
            // particles' contribution
            const float2 p = inc ? df_sub(phi_prev[pb + r[j]], d[j]) : d[j];
            phi_cur[pb + r[j]] = p;
            const float pf = p.x + p.y;
            const float dx = u[j].x - wx, dy = u[j].y - wy, dz = u[j].z - wz;
            const float ek = 0.5f * (dx * dx + dy * dy + dz * dz);
            const float e = ek - gfac * pf;
            const bool keep = !(e > 0.f);
            keepf[pb + r[j]] = keep ? 1 : 0;
            gone[slot] = keep ? 0 : 1;
            if (keep) {
                ++kept;
                two_sum_acc(ek_s, ek_c, u[j].w * ek);
                two_sum_acc(ep_s, ep_c, u[j].w * pf);
                if (phi_out) phi_out[pidx[pb + r[j]]] = df_to_double(p);
            } else {
                ++removed;
                const int i = pidx[pb + r[j]];
                bound[i] = 0;
                if (phi_out) phi_out[i] = 0.0;
            }
        }
        // block sums: counts exactly, energies in double-float (warp tree, then warps in order)
        float2 ekv = df_warp_sum(df_from_acc(ek_s, ek_c));
        float2 epv = df_warp_sum(df_from_acc(ep_s, ep_c));
        int kc = kept, rc = removed;
        for (int o = 16; o > 0; o >>= 1) {
            kc += __shfl_down_sync(0xffffffffu, kc, o);
            rc += __shfl_down_sync(0xffffffffu, rc, o);
        }
        if (lane == 0) {
            se[0][w] = ekv;
            se[1][w] = epv;
            sc[0][w] = kc;
            sc[1][w] = rc;
        }
        __syncthreads();
        int nrem = 0;
        for (int k = 0; k < kSegThreads / 32; ++k) nrem += sc[1][k];
        if (w == 0) {
            // the removed particles in slot order (32 slots per step)
            int base = 0;
            if (nrem > 0)
                for (int s0 = 0; s0 < kSeg; s0 += 32) {
                    const bool g = gone[s0 + lane];
                    const unsigned bal = __ballot_sync(0xffffffffu, g);
                    if (g) rlist[base + __popc(bal & ((1u << lane) - 1u))] = pidx[pb + sl * kSeg + s0 + lane];
                    base += __popc(bal);
                }
            __syncwarp();
            double a[7] = {0, 0, 0, 0, 0, 0, 0};
            for (int k = lane; k < nrem; k += 32) {
                const int i = rlist[k];
                const double mi = m[i];
                a[0] += mi;
                a[1] += mi * x[i];
                a[2] += mi * y[i];
                a[3] += mi * z[i];
                a[4] += mi * vx[i];
                a[5] += mi * vy[i];
                a[6] += mi * vz[i];
            }
            if (nrem > 0)
#pragma unroll
                for (int k = 0; k < 7; ++k) a[k] = warp_sum(a[k]);
            if (lane == 0) {
                SegDF o;
                o.removed = nrem;
                o.kept = 0;
                float2 e0 = make_float2(0.f, 0.f), e1 = make_float2(0.f, 0.f);
                for (int k = 0; k < kSegThreads / 32; ++k) {
                    o.kept += sc[0][k];
                    e0 = df_add(e0, se[0][k]);
                    e1 = df_add(e1, se[1][k]);
                }
                o.ekin = e0;
                o.epot = e1;
                o.rm = a[0]; o.rmx = a[1]; o.rmy = a[2]; o.rmz = a[3];
                o.rmvx = a[4]; o.rmvy = a[5]; o.rmvz = a[6];
                seg_sums[seg] = o;
            }
        }
        __syncthreads();   // the shared arrays are reused by the next segment
    }
}

// One warp per active ordered halo after the energy pass (FP32 path): segment sums in a fixed
// order; survivors / removed before each segment (seg_pre); removals, pass count, energies;
// the halo's FP64 mass and sums of m x, m v less the removed particles' (a halo left empty
// is set to zero exactly), its centre, bulk velocity and the FP32 bulk-velocity offset for
// the next pass.  A halo whose pass removed nothing becomes inactive.
__global__ void ub_finalize_df_kernel(int nh, const int *__restrict__ order, const int *__restrict__ sstart,
                                      const SegDF *__restrict__ seg_sums, double gfac, HaloState *hs,
                                      int2 *__restrict__ seg_pre) {
    const int q = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (q >= nh) return;
    const int h = order[q];
    if (!hs[h].active) return;
    const int s0 = sstart[q], s1 = sstart[q + 1];
    float2 ek = make_float2(0.f, 0.f), ep = make_float2(0.f, 0.f);
    double a[7] = {0, 0, 0, 0, 0, 0, 0};
    int keep_run = 0, rem_run = 0;
    for (int b0 = s0; b0 < s1; b0 += 32) {
        const int sg = b0 + lane;
        const bool ok = sg < s1;
        const int nrem = ok ? seg_sums[sg].removed : 0;
        const int nkeep = ok ? seg_sums[sg].kept : 0;
        const int ri = warp_incl_scan(nrem, lane), ki = warp_incl_scan(nkeep, lane);
        if (ok) seg_pre[sg] = make_int2(keep_run + ki - nkeep, rem_run + ri - nrem);
        keep_run += __shfl_sync(0xffffffffu, ki, 31);
        rem_run += __shfl_sync(0xffffffffu, ri, 31);
        if (ok) {
            const SegDF &g = seg_sums[sg];
            ek = df_add(ek, g.ekin);
            ep = df_add(ep, g.epot);
            if (g.removed > 0) {
                a[0] += g.rm; a[1] += g.rmx; a[2] += g.rmy; a[3] += g.rmz;
                a[4] += g.rmvx; a[5] += g.rmvy; a[6] += g.rmvz;
            }
        }
    }
    ek = df_warp_sum(ek);
    ep = df_warp_sum(ep);
    if (rem_run > 0)
#pragma unroll
        for (int k = 0; k < 7; ++k) a[k] = warp_sum(a[k]);
    if (lane == 0) {
        HaloState &o = hs[h];
        o.nprev = o.nb;
        o.removed = rem_run;
        o.nrem = rem_run;
        o.iter += 1;
        o.ekin = df_to_double(ek);
        o.epot = -0.5 * gfac * df_to_double(ep);
        if (rem_run == 0) {
            o.active = 0;
        } else {
            o.nb = keep_run;
            if (keep_run == 0) {
                o.M = o.sx = o.sy = o.sz = o.px = o.py = o.pz = 0.0;
            } else {
                o.M -= a[0];
                o.sx -= a[1]; o.sy -= a[2]; o.sz -= a[3];
                o.px -= a[4]; o.py -= a[5]; o.pz -= a[6];
            }
            const double M = o.M;
            if (M > 0) {
                o.cx = o.sx / M; o.cy = o.sy / M; o.cz = o.sz / M;
                o.vx = o.px / M; o.vy = o.py / M; o.vz = o.pz / M;
            } else {
                o.cx = o.cy = o.cz = o.vx = o.vy = o.vz = 0.0;
            }
            o.wx = (float)(o.vx - o.v0x);
            o.wy = (float)(o.vy - o.v0y);
            o.wz = (float)(o.vz - o.v0z);
        }
    }
}

// Per segment of a halo that stays active (FP32 path): survivors' packed position, velocity
// offset, index and potential copied in order into the other buffers, removed particles'
// packed positions into the next pass's source list; the halo's last segment pads both.
__global__ void __launch_bounds__(kSegThreads) ub_compact_df_kernel(
    const int *__restrict__ sstart, const int *__restrict__ sown, const int4 *__restrict__ idesc,
    const int *__restrict__ nsegs, const int64_t *__restrict__ poff, const HaloState *__restrict__ hs,
    const unsigned char *__restrict__ keepf, const int2 *__restrict__ seg_pre, const float4 *__restrict__ pk_in,
    const float4 *__restrict__ pv_in, const int *__restrict__ pidx_in, const float2 *__restrict__ phi_cur,
    float4 *__restrict__ pk_out, float4 *__restrict__ pv_out, int *__restrict__ pidx_out,
    float2 *__restrict__ phi_next, float4 *__restrict__ removed) {
    __shared__ int wcount[kSegThreads / 32], wrem[kSegThreads / 32];
    const int nseg_all = *nsegs;
    for (int seg = blockIdx.x; seg < nseg_all; seg += gridDim.x) {
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        const int q = sown[seg];
        const int h = idesc[q].x;
        if (!hs[h].active) continue;   // converged this pass: its packed slots are not read again
        const int s0 = sstart[q], sl = seg - s0, nseg = sstart[q + 1] - s0;
        const int nb = hs[h].nprev;
        const int64_t pb = poff[h];
        const int2 pre = seg_pre[seg];
        int running = pre.x, rrunning = pre.y;
        const int rend = min(nb, (sl + 1) * kSeg);
        for (int r0 = sl * kSeg; r0 < rend; r0 += kSegThreads) {
            const int r = r0 + threadIdx.x;
            const bool valid = r < rend;
            const bool keep = valid && keepf[pb + r];
            const bool gone = valid && !keep;
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            const unsigned bgone = __ballot_sync(0xffffffffu, gone);
            if (lane == 0) {
                wcount[w] = __popc(bal);
                wrem[w] = __popc(bgone);
            }
            __syncthreads();
            int rank = running, rrank = rrunning, tot = 0, trem = 0;
#pragma unroll
            for (int k = 0; k < kSegThreads / 32; ++k) {
                if (k < w) {
                    rank += wcount[k];
                    rrank += wrem[k];
                }
                tot += wcount[k];
                trem += wrem[k];
            }
            rank += __popc(bal & ((1u << lane) - 1u));
            rrank += __popc(bgone & ((1u << lane) - 1u));
            if (keep) {
                pk_out[pb + rank] = pk_in[pb + r];
                pv_out[pb + rank] = pv_in[pb + r];
                pidx_out[pb + rank] = pidx_in[pb + r];
                phi_next[pb + rank] = phi_cur[pb + r];
            } else if (gone) {
                removed[pb + rrank] = pk_in[pb + r];
            }
            running += tot;
            rrunning += trem;
            __syncthreads();
        }
        if (sl == nseg - 1) {   // the halo's last segment pads after the survivors and the removed
            const float4 f = make_float4(kFar, kFar, kFar, 0.f);
            const int nkeep = running, nrem = rrunning;
            for (int r = nkeep + threadIdx.x; r < ((nkeep + 31) & ~31); r += kSegThreads) {
                pk_out[pb + r] = f;
                pv_out[pb + r] = make_float4(0.f, 0.f, 0.f, 0.f);
                pidx_out[pb + r] = -1;
            }
            for (int r = nrem + threadIdx.x; r < ((nrem + 31) & ~31); r += kSegThreads) removed[pb + r] = f;
        }
        __syncthreads();   // the shared arrays are reused by the next segment
    }
}

// Plain FP64 pair kernel for one halo (targets = sources = its packed slots).
__global__ void __launch_bounds__(256) ub_pair_f64_kernel(const double4 *__restrict__ pk, int nb, double eps2,
                                                          double *__restrict__ phi) {
    __shared__ double4 sb[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double4 p = i < nb ? pk[i] : make_double4(0, 0, 0, 0);
    double acc = 0.0;
    for (int j0 = 0; j0 < nb; j0 += 256) {
        __syncthreads();
        if (j0 + threadIdx.x < nb) sb[threadIdx.x] = pk[j0 + threadIdx.x];
        __syncthreads();
        const int cnt = min(256, nb - j0);
        for (int k = 0; k < cnt; ++k) {
            if (j0 + k == i) continue;
            const double4 q = sb[k];
            const double dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
            acc = fma(q.w, rsqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)))), acc);
        }
    }
    if (i < nb) phi[i] = acc;
}

__global__ void ub_output_kernel(int nh, const HaloState *__restrict__ hs, double *__restrict__ out) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x) {
        const HaloState s = hs[h];
        double *o = out + (int64_t)h * HALMA_UB_NFIELDS;
        o[HALMA_UB_MASS] = s.M;
        o[HALMA_UB_CX] = s.cx; o[HALMA_UB_CY] = s.cy; o[HALMA_UB_CZ] = s.cz;
        o[HALMA_UB_VX] = s.vx; o[HALMA_UB_VY] = s.vy; o[HALMA_UB_VZ] = s.vz;
        o[HALMA_UB_NBOUND] = (double)s.nb;
        o[HALMA_UB_ITER] = (double)s.iter;
        o[HALMA_UB_EKIN] = s.ekin;
        o[HALMA_UB_EPOT] = s.epot;
    }
}

// The passes are captured in chunks of kPassChunk (the first chunk also holds the reduction
// and packing); one graph per chunk start, all cached for the same problem shape.
constexpr int kPassChunk = 8;
struct GraphCache {
    struct Entry {
        cudaGraphExec_t exec = nullptr;
        int64_t nodes = 0;
    };
    std::vector<Entry> chunks;   // by chunk start / kPassChunk
    std::vector<uintptr_t> key;
    cudaStream_t capture_stream = nullptr;
    int capture_device = -1;
};
GraphCache &graph_cache() {
    static GraphCache g;
    return g;
}

// Number of haloes still active after a chunk of passes (the host stops replaying at 0).
__global__ void ub_active_kernel(int nh, const HaloState *__restrict__ hs, int *__restrict__ count) {
    int a = 0;
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x) a += hs[h].active;
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0 && a) atomicAdd(count, a);
}

}  // namespace

Profile &profile() {
    static Profile p;
    return p;
}

static TileTable &tile_table_ref() {
    // default until the autotuner's table is loaded: 1 chunk of targets for haloes of up to
    // 32 bound particles, 2 up to 64, 4 above
    static TileTable t = {3, {32, 64, 0x7fffffff}, {1, 2, 4}, 4096};
    return t;
}

TileTable tile_table() { return tile_table_ref(); }

int Profile::fof_mark(int stage, cudaStream_t st) {
    if (!enabled) return HALMA_OK;
    if (!fev[stage]) HALMA_CUDA(cudaEventCreate(&fev[stage]));
    HALMA_CUDA(cudaEventRecord(fev[stage], st));
    return HALMA_OK;
}

int Profile::ensure_events(int k) {
    while ((int)ev0.size() < k) {
        cudaEvent_t a, b, c;
        HALMA_CUDA(cudaEventCreate(&a));
        HALMA_CUDA(cudaEventCreate(&b));
        HALMA_CUDA(cudaEventCreate(&c));
        ev0.push_back(a);
        ev1.push_back(b);
        evm.push_back(c);
    }
    return HALMA_OK;
}

int sym_block_count(int nb) { return (nb + kSymBlock - 1) / kSymBlock; }

// Self-potential of nb particles packed as float4 (x, y, z, m), every pair evaluated once for
// both particles by the symmetric block kernel: part[b * npad + r] (npad = nb rounded up to
// 32) receives the double-float sum over the sources of block b of m_j (r^2 + eps2)^-1/2,
// j != r, for b < sym_block_count(nb).  scratch: 512 bytes of device memory for the
// description of the single work list.
int sym_self_potential_device(const float4 *pk, int nb, float eps2, float2 *part, void *scratch, cudaStream_t st) {
    if (nb <= 0) return HALMA_OK;
    if (nb > 65535 * kSymBlock) return fail(HALMA_ERR_CAPACITY, "at most %d particles", 65535 * kSymBlock);
    const int64_t B = sym_block_count(nb);
    struct Desc {
        HaloState hs;
        int64_t poff[2], qoff[2];
        int4 idesc;
        int ystart[2];
        int cnt[8];
    } d{};
    static_assert(sizeof(Desc) <= 512, "work description exceeds its scratch");
    d.hs.nb = nb;
    d.hs.active = 1;
    d.poff[1] = ((int64_t)nb + 31) / 32 * 32;
    d.idesc = make_int4(0, kSymT, 1, (int)B);
    d.ystart[1] = (int)(B * (B + 1) / 2);
    d.cnt[3] = d.ystart[1];
    HALMA_CUDA(cudaMemcpyAsync(scratch, &d, sizeof(Desc), cudaMemcpyHostToDevice, st));
    Desc *dd = static_cast<Desc *>(scratch);
    constexpr int kSymSmem = kSymBlock * (int)sizeof(float4) + kSymWarps * kSymBlock * (int)sizeof(float);
    HALMA_CUDA(cudaFuncSetAttribute(ub_pair_sym_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSymSmem));
    int bps = 0;
    HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ub_pair_sym_kernel, 128, kSymSmem));
    const int grid = (int)std::min<int64_t>((int64_t)device_sm_count() * std::max(bps, 1), d.cnt[3]);
    HALMA_LAUNCH(ub_pair_sym_kernel, grid, 128, kSymSmem, st, pk, dd->poff, dd->qoff, &dd->hs, 1, dd->ystart,
                 &dd->idesc, dd->cnt, dd->cnt + 4, eps2, part);
    return HALMA_OK;
}

// Device-array implementation shared by halma_unbind_batched and the pipeline.
int unbind_device(int64_t n, int nh, const int64_t *d_off, const int64_t *h_off, const double *x, const double *y,
                  const double *z, const double *vx, const double *vy, const double *vz, const double *m,
                  const halma_unbind_params &p, unsigned char *bound, double *phi_out, double *halo_out,
                  cudaStream_t st, cudaEvent_t vel_ready) {
    const TileTable tab = tile_table();
    const bool f64 = p.precision == HALMA_UNBIND_FP64;
    // source slice length (a multiple of 32); the FP64 path sums a halo in one piece
    const int slice_len = f64 ? (1 << 30) : tab.slice;
    // host-side plan: padded slot offsets, per-slice partial-sum offsets, size order
    std::vector<int64_t> poff(nh + 1), qoff(nh + 1);
    std::vector<int> order(nh);
    poff[0] = 0;
    qoff[0] = 0;
    int64_t segcap = 0;   // energy segments at most (initial sizes)
    std::vector<int> cstart(nh + 1), chunk_h;   // member chunks of kSeg (reduce and first pack)
    for (int h = 0; h < nh; ++h) {
        const int64_t c = h_off[h + 1] - h_off[h];
        cstart[h] = (int)chunk_h.size();
        for (int64_t k = 0; k < (c + kSeg - 1) / kSeg; ++k) chunk_h.push_back(h);
        const int64_t npad = ((c + 31) / 32) * 32;
        int64_t nsl = std::max<int64_t>(1, (c + slice_len - 1) / slice_len);
        if (!f64 && c > kSymBlock) nsl = std::max<int64_t>(nsl, (c + kSymBlock - 1) / kSymBlock);   // symmetric
        poff[h + 1] = poff[h] + npad;
        qoff[h + 1] = qoff[h] + npad * nsl;
        segcap += std::max<int64_t>(1, (c + kSeg - 1) / kSeg);
    }
    cstart[nh] = (int)chunk_h.size();
    const int nchunks = (int)chunk_h.size();
    if (segcap >= (1ll << 31)) return fail(HALMA_ERR_CAPACITY, "too many energy segments");
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (h_off[a + 1] - h_off[a]) > (h_off[b + 1] - h_off[b]);
    });
    const int64_t P = std::max<int64_t>(poff[nh], 32);
    const int64_t Q = std::max<int64_t>(qoff[nh], 32);
    Layout L;
    const size_t o_hs = L.add(sizeof(HaloState) * (size_t)std::max(nh, 1));
    const size_t o_poff = L.add(sizeof(int64_t) * (nh + 1));
    const size_t o_qoff = L.add(sizeof(int64_t) * (nh + 1));
    const size_t o_order = L.add(sizeof(int) * std::max(nh, 1));
    const size_t vsz = f64 ? sizeof(double4) : sizeof(float4);
    const size_t o_pk = L.add(vsz * P), o_pk2 = L.add(vsz * P);       // packed slots, double-buffered
    const size_t o_pidx = L.add(sizeof(int) * P), o_pidx2 = L.add(sizeof(int) * P);
    const size_t o_keep = L.add(P);
    const size_t o_rk = L.add(vsz * P);                               // removed particles' slots
    const size_t o_phic = L.add(sizeof(double) * P), o_phin = L.add(sizeof(double) * P);
    const size_t o_phi = L.add(sizeof(double) * Q);
    const size_t o_istart = L.add(sizeof(int) * (nh + 1));
    const size_t o_sstart = L.add(sizeof(int) * (nh + 1));
    const size_t o_idesc = L.add(sizeof(int4) * std::max(nh, 1));
    const size_t o_ssum = L.add(std::max(sizeof(double) * kSegSums, sizeof(SegDF)) * segcap);
    const size_t o_pv = L.add(f64 ? 0 : sizeof(float4) * P), o_pv2 = L.add(f64 ? 0 : sizeof(float4) * P);
    const size_t o_sown = L.add(sizeof(int) * segcap);
    const size_t o_spre = L.add(sizeof(int2) * segcap);
    const size_t o_cst = L.add(sizeof(int) * (nh + 1));
    const size_t o_chh = L.add(sizeof(int) * std::max(nchunks, 1));
    const size_t o_rpart = L.add(sizeof(double) * kRedSums * std::max(nchunks, 1));
    const size_t o_cnt = L.add(64);
    const size_t o_pairs = L.add(sizeof(unsigned long long) * 2 * p.max_iter);
    const size_t o_ystart = L.add(sizeof(int) * (nh + 1));
    const size_t o_off = d_off ? 0 : L.add(sizeof(int64_t) * (nh + 1));
    const size_t o_icnt = L.add(sizeof(int4) * std::max(nh, 1)), o_ipre = L.add(sizeof(int4) * std::max(nh, 1));
    const size_t iscan_bytes = exclusive_sum_int3_bytes(std::max(nh, 1));
    const size_t o_iscan = L.add(iscan_bytes);
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    auto *hs = at<HaloState>(base, o_hs);
    auto *dpoff = at<int64_t>(base, o_poff);
    auto *dqoff = at<int64_t>(base, o_qoff);
    auto *dorder = at<int>(base, o_order);
    int *pidxb[2] = {at<int>(base, o_pidx), at<int>(base, o_pidx2)};
    auto *keepf = at<unsigned char>(base, o_keep);
    auto *phic = at<double>(base, o_phic), *phin = at<double>(base, o_phin);
    // incremental passes subtract the removed particles' potential instead of recomputing
    const bool incremental = !(p.flags & HALMA_UNBIND_FULL_RECOMPUTE);
    auto *phi = at<double>(base, o_phi);
    auto *istart = at<int>(base, o_istart);
    auto *sstart = at<int>(base, o_sstart);
    auto *idesc = at<int4>(base, o_idesc);
    auto *ssum = at<double>(base, o_ssum);
    auto *sown = at<int>(base, o_sown);
    auto *segpre = at<int2>(base, o_spre);
    auto *dcst = at<int>(base, o_cst);
    auto *dchh = at<int>(base, o_chh);
    auto *rpart = at<double>(base, o_rpart);
    int *cnt = at<int>(base, o_cnt);   // [0] nitems [1] counter [2] energy segments
    const int sgrid = (int)segcap;
    auto *dpairs = at<unsigned long long>(base, o_pairs);
    auto *ystart = at<int>(base, o_ystart);
    Profile &prof = profile();
    const bool profiling = prof.enabled;
    if (profiling) {
        HALMA_TRY(prof.ensure_events(p.max_iter));
        HALMA_CUDA(cudaMemsetAsync(dpairs, 0, sizeof(unsigned long long) * 2 * p.max_iter, st));
    }
    const int64_t *off = d_off;
    if (!d_off) {
        int64_t *o = at<int64_t>(base, o_off);
        HALMA_CUDA(cudaMemcpyAsync(o, h_off, sizeof(int64_t) * (nh + 1), cudaMemcpyHostToDevice, st));
        off = o;
    }
    HALMA_CUDA(cudaMemcpyAsync(dpoff, poff.data(), sizeof(int64_t) * (nh + 1), cudaMemcpyHostToDevice, st));
    HALMA_CUDA(cudaMemcpyAsync(dqoff, qoff.data(), sizeof(int64_t) * (nh + 1), cudaMemcpyHostToDevice, st));
    HALMA_CUDA(cudaMemcpyAsync(dorder, order.data(), sizeof(int) * nh, cudaMemcpyHostToDevice, st));
    HALMA_CUDA(cudaMemcpyAsync(dcst, cstart.data(), sizeof(int) * (nh + 1), cudaMemcpyHostToDevice, st));
    if (nchunks > 0)
        HALMA_CUDA(cudaMemcpyAsync(dchh, chunk_h.data(), sizeof(int) * nchunks, cudaMemcpyHostToDevice, st));
    const int fgrid = grid_for((int64_t)nh * 32, 256);   // one warp per halo
    // the pass's work list (count, scan, fill; see ub_items_count_kernel)
    auto *icount = at<int4>(base, o_icnt), *ipre = at<int4>(base, o_ipre);
    void *iscan_tmp = at<void>(base, o_iscan);
    const int igrid = std::min(grid_for(nh, 256), device_sm_count() * 4);
    auto items = [&](cudaStream_t rs, int inc, int sym_ok, unsigned long long *pairs) -> int {
        if (pairs) HALMA_CUDA(cudaMemsetAsync(pairs, 0, 2 * sizeof(unsigned long long), rs));
        HALMA_LAUNCH(ub_items_count_kernel, igrid, 256, 0, rs, nh, dorder, hs, tab, slice_len, inc, sym_ok, icount,
                     idesc, pairs);
        HALMA_TRY(exclusive_sum_int3(iscan_tmp, iscan_bytes, icount, ipre, nh, rs));
        HALMA_LAUNCH(ub_items_fill_kernel, igrid, 256, 0, rs, nh, icount, ipre, istart, ystart, sstart, sown, cnt);
        return HALMA_OK;
    };
    // FP64 bound mass, centre and bulk velocity per halo (active ones, or all with force);
    // part as in ub_reduce_seg_kernel (the halo state is final after parts 1 and 2 in turn)
    auto reduce = [&](cudaStream_t rs, int force, int part = 0) -> int {
        if (nchunks > 0) {
            if (part == 1)
                HALMA_LAUNCH(ub_reduce_seg_kernel<1>, nchunks, kSegThreads, 0, rs, off, dcst, dchh, x, y, z, vx, vy,
                             vz, m, bound, hs, force, rpart);
            else if (part == 2)
                HALMA_LAUNCH(ub_reduce_seg_kernel<2>, nchunks, kSegThreads, 0, rs, off, dcst, dchh, x, y, z, vx, vy,
                             vz, m, bound, hs, force, rpart);
            else
                HALMA_LAUNCH(ub_reduce_seg_kernel<0>, nchunks, kSegThreads, 0, rs, off, dcst, dchh, x, y, z, vx, vy,
                             vz, m, bound, hs, force, rpart);
        }
        HALMA_LAUNCH(ub_reduce_fin_kernel, fgrid, 256, 0, rs, nh, dcst, rpart, force, hs);
        return HALMA_OK;
    };
    const double gfac = p.G * p.factor_v * p.factor_v;
    const float eps2 = (float)(p.eps * p.eps);
    HALMA_LAUNCH(ub_init_kernel, std::min(device_sm_count() * 8, grid_for(std::max<int64_t>(n, nh), 256)), 256, 0, st,
                 n, bound, nh, hs);
    if (phi_out) HALMA_CUDA(cudaMemsetAsync(phi_out, 0, sizeof(double) * n, st));

    if (!f64) {
        float4 *pkb[2] = {at<float4>(base, o_pk), at<float4>(base, o_pk2)};
        float4 *pvb[2] = {at<float4>(base, o_pv), at<float4>(base, o_pv2)};
        auto *part2 = reinterpret_cast<float2 *>(phi);   // double-float partials and potentials
        auto *phic2 = reinterpret_cast<float2 *>(phic), *phin2 = reinterpret_cast<float2 *>(phin);
        auto *sdf = reinterpret_cast<SegDF *>(ssum);
        const float gfac_f = (float)gfac;
        int bps = 0;
        HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ub_pair_kernel, 256, 0));
        const int pgrid = device_sm_count() * std::max(bps, 1);
        constexpr int kSymSmem = kSymBlock * (int)sizeof(float4) + kSymWarps * kSymBlock * (int)sizeof(float);
        HALMA_CUDA(cudaFuncSetAttribute(ub_pair_sym_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSymSmem));
        HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ub_pair_sym_kernel, 128, kSymSmem));
        const int ygrid = device_sm_count() * std::max(bps, 1);
        // the end-of-pass kernels loop over the pass's energy segments with one wave of blocks
        // (a launch of one block per possible segment cost ~30 us even when few were active)
        HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ub_energy_df_kernel, kSegThreads, 0));
        const int egrid = std::min(sgrid, device_sm_count() * std::max(bps, 1));
        HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ub_compact_df_kernel, kSegThreads, 0));
        const int cgrid = std::min(sgrid, device_sm_count() * std::max(bps, 1));
        auto record = [&](cudaStream_t rs, int it0, int it1) -> int {
            // first pass: centre of mass and packing into buffer 0; every pass then compacts
            // its survivors into the other buffer and sets the next pass's halo state
            // With vel_ready, the velocities may still be arriving: the first pass's pair
            // kernels start from the positions and masses, and the velocity sums and packed
            // velocities follow once vel_ready has fired (an external wait: a node of the
            // captured graph), before the first energy kernel.
            if (it0 == 0) {
                HALMA_TRY(reduce(rs, 0, vel_ready ? 1 : 0));
                if (nchunks > 0)
                    HALMA_LAUNCH(ub_pack_kernel<float4>, nchunks, kSegThreads, 0, rs, off, dpoff, dcst, dchh, x, y, z,
                                 m, vx, vy, vz, hs, pkb[0], vel_ready ? nullptr : pvb[0], pidxb[0]);
            }
            float4 *rk = at<float4>(base, o_rk);
            for (int it = it0; it < it1; ++it) {
                const int a = it & 1, b = a ^ 1;
                const int inc = (it > 0 && incremental) ? 1 : 0;
                HALMA_TRY(items(rs, inc, 1, profiling ? dpairs + 2 * it : nullptr));
                // External: captured as an event-record node, so the replay records it
                if (profiling) HALMA_CUDA(cudaEventRecordWithFlags(prof.ev0[it], rs, cudaEventRecordExternal));
                // full passes: the big haloes' block pairs first (the longest items), then the
                // tiles of the small ones; incremental passes have only tiles
                if (!inc)
                    HALMA_LAUNCH(ub_pair_sym_kernel, ygrid, 128, kSymSmem, rs, pkb[a], dpoff, dqoff, hs, nh, ystart,
                                 idesc, cnt, cnt + 4, eps2, part2);
                if (profiling) HALMA_CUDA(cudaEventRecordWithFlags(prof.evm[it], rs, cudaEventRecordExternal));
                HALMA_LAUNCH(ub_pair_kernel, pgrid, 256, 0, rs, pkb[a], rk, inc, dpoff, dqoff, hs, nh, istart, idesc,
                             cnt, cnt + 1, eps2, slice_len / 32, part2);
                if (profiling) HALMA_CUDA(cudaEventRecordWithFlags(prof.ev1[it], rs, cudaEventRecordExternal));
                if (it == 0 && vel_ready) {
                    HALMA_CUDA(cudaStreamWaitEvent(rs, vel_ready, cudaEventWaitExternal));
                    HALMA_TRY(reduce(rs, 0, 2));
                    if (nchunks > 0)
                        HALMA_LAUNCH(ub_pack_kernel<float4>, nchunks, kSegThreads, 0, rs, off, dpoff, dcst, dchh, x, y,
                                     z, m, vx, vy, vz, hs, (float4 *)nullptr, pvb[0], (int *)nullptr);
                }
                HALMA_LAUNCH(ub_energy_df_kernel, egrid, kSegThreads, 0, rs, sstart, sown, idesc, cnt + 2, dpoff, dqoff,
                             inc, pidxb[a], pvb[a], part2, phin2, phic2, x, y, z, vx, vy, vz, m, gfac_f, hs, bound,
                             phi_out, keepf, sdf);
                HALMA_LAUNCH(ub_finalize_df_kernel, fgrid, 256, 0, rs, nh, dorder, sstart, sdf, gfac, hs, segpre);
                HALMA_LAUNCH(ub_compact_df_kernel, cgrid, kSegThreads, 0, rs, sstart, sown, idesc, cnt + 2, dpoff, hs,
                             keepf, segpre, pkb[a], pvb[a], pidxb[a], phic2, pkb[b], pvb[b], pidxb[b], phin2, rk);
            }
            HALMA_CUDA(cudaMemsetAsync(cnt + 6, 0, sizeof(int), rs));
            HALMA_LAUNCH(ub_active_kernel, std::min(grid_for(nh, 256), 64), 256, 0, rs, nh, hs, cnt + 6);
            return HALMA_OK;
        };
        int passes_run = p.max_iter;
        if (p.use_graph) {
            std::vector<uintptr_t> key = {(uintptr_t)base, (uintptr_t)off, (uintptr_t)x, (uintptr_t)y, (uintptr_t)z,
                                          (uintptr_t)vx, (uintptr_t)vy, (uintptr_t)vz, (uintptr_t)m,
                                          (uintptr_t)bound, (uintptr_t)phi_out, (uintptr_t)n, (uintptr_t)nh,
                                          (uintptr_t)p.max_iter, (uintptr_t)st};
            uint64_t eb = 0, gb = 0;
            memcpy(&eb, &eps2, sizeof(float));
            memcpy(&gb, &gfac, sizeof(double));
            key.push_back((uintptr_t)eb);
            key.push_back((uintptr_t)gb);
            key.insert(key.end(), poff.begin(), poff.end());
            key.push_back((uintptr_t)current_device());
            key.push_back((uintptr_t)profiling);
            key.push_back((uintptr_t)dpairs);
            key.push_back((uintptr_t)tab.n);
            key.push_back((uintptr_t)slice_len);
            key.push_back((uintptr_t)incremental);
            key.push_back((uintptr_t)nchunks);
            key.push_back((uintptr_t)vel_ready);
            for (int c = 0; c < tab.n; ++c) {
                key.push_back((uintptr_t)tab.upper[c]);
                key.push_back((uintptr_t)tab.t[c]);
            }
            GraphCache &gc = graph_cache();
            if (gc.key != key) {
                for (auto &e : gc.chunks)
                    if (e.exec) cudaGraphExecDestroy(e.exec);
                gc.chunks.clear();
                gc.key = key;
            }
            // capture on a private stream (the legacy default stream cannot be captured)
            if (!gc.capture_stream || gc.capture_device != current_device()) {
                HALMA_CUDA(cudaStreamCreateWithFlags(&gc.capture_stream, cudaStreamNonBlocking));
                gc.capture_device = current_device();
            }
            const int nchunk = (p.max_iter + kPassChunk - 1) / kPassChunk;
            gc.chunks.resize(nchunk);
            passes_run = 0;
            for (int ci = 0; ci < nchunk; ++ci) {
                const int it0 = ci * kPassChunk, it1 = std::min(p.max_iter, it0 + kPassChunk);
                GraphCache::Entry &ge = gc.chunks[ci];
                if (!ge.exec) {
                    cudaGraph_t graph = nullptr;
                    HALMA_CUDA(cudaStreamBeginCapture(gc.capture_stream, cudaStreamCaptureModeThreadLocal));
                    const int64_t before = halma_kernel_launch_count();
                    int s = record(gc.capture_stream, it0, it1);
                    cudaError_t ce = cudaStreamEndCapture(gc.capture_stream, &graph);
                    if (s != HALMA_OK) {
                        if (graph) cudaGraphDestroy(graph);
                        return s;
                    }
                    HALMA_CUDA(ce);
                    cudaError_t ie = cudaGraphInstantiate(&ge.exec, graph, 0);
                    cudaGraphDestroy(graph);
                    HALMA_CUDA(ie);
                    ge.nodes = halma_kernel_launch_count() - before;
                    add_launches(-ge.nodes);   // counted again at every replay below
                }
                HALMA_CUDA(cudaGraphLaunch(ge.exec, st));
                add_launches(ge.nodes);
                passes_run = it1;
                if (it1 >= p.max_iter) break;
                int active = 0;
                HALMA_CUDA(cudaMemcpyAsync(&active, cnt + 6, sizeof(int), cudaMemcpyDeviceToHost, st));
                HALMA_CUDA(cudaStreamSynchronize(st));
                if (active == 0) break;
            }
        } else {
            HALMA_TRY(record(st, 0, p.max_iter));
        }
        // the halo state already holds the final bound set's mass, centre and bulk velocity
        if (profiling) {
            std::vector<unsigned long long> hp(2 * p.max_iter);
            HALMA_CUDA(cudaMemcpyAsync(hp.data(), dpairs, sizeof(unsigned long long) * 2 * p.max_iter,
                                       cudaMemcpyDeviceToHost, st));
            HALMA_CUDA(cudaStreamSynchronize(st));
            prof.passes.clear();
            for (int it = 0; it < passes_run; ++it) {
                float ms = 0.f, sms = 0.f;
                HALMA_CUDA(cudaEventElapsedTime(&ms, prof.ev0[it], prof.ev1[it]));
                HALMA_CUDA(cudaEventElapsedTime(&sms, prof.ev0[it], prof.evm[it]));
                prof.passes.push_back({(double)hp[2 * it], (double)ms, (double)hp[2 * it + 1], (double)sms});
            }
        }
    } else {
        // plain FP64 path: per pass, one pair launch per active halo, host checks convergence
        double4 *pkb[2] = {at<double4>(base, o_pk), at<double4>(base, o_pk2)};
        std::vector<HaloState> hh(nh);
        HALMA_TRY(reduce(st, 0));
        if (nchunks > 0)
            HALMA_LAUNCH(ub_pack_kernel<double4>, nchunks, kSegThreads, 0, st, off, dpoff, dcst, dchh, x, y, z, m, vx,
                         vy, vz, hs, pkb[0], nullptr, pidxb[0]);
        double4 *rk = at<double4>(base, o_rk);
        for (int it = 0; it < p.max_iter; ++it) {
            const int a = it & 1, b = a ^ 1;
            HALMA_TRY(items(st, 0, 0, nullptr));
            HALMA_CUDA(cudaMemcpyAsync(hh.data(), hs, sizeof(HaloState) * nh, cudaMemcpyDeviceToHost, st));
            HALMA_CUDA(cudaStreamSynchronize(st));
            int any = 0;
            for (int h = 0; h < nh; ++h) {
                if (!hh[h].active || hh[h].nb == 0) continue;
                any = 1;
                HALMA_LAUNCH(ub_pair_f64_kernel, grid_for(hh[h].nb, 256), 256, 0, st, pkb[a] + poff[h], hh[h].nb,
                             p.eps * p.eps, phi + poff[h]);
            }
            if (!any) break;
            HALMA_LAUNCH(ub_energy_seg_kernel<double4>, sgrid, kSegThreads, 0, st, sstart, sown, idesc, cnt + 2, dpoff,
                         dqoff, 0, pidxb[a], phi, phin, phic, vx, vy, vz, m, gfac, hs, bound, phi_out, keepf,
                         ssum);
            HALMA_LAUNCH(ub_finalize_kernel, fgrid, 256, 0, st, nh, dorder, sstart, ssum, gfac, hs, segpre);
            HALMA_LAUNCH(ub_compact_seg_kernel<double4>, sgrid, kSegThreads, 0, st, sstart, sown, idesc, cnt + 2, dpoff,
                         hs, keepf, segpre, pkb[a], pidxb[a], phic, pkb[b], pidxb[b], phin, rk);
        }
        HALMA_TRY(reduce(st, 1));
    }
    if (halo_out) HALMA_LAUNCH(ub_output_kernel, grid_for(nh, 256), 256, 0, st, nh, hs, halo_out);
    return HALMA_OK;
}

}  // namespace halma

using namespace halma;

extern "C" int halma_unbind_batched(int64_t n, int64_t n_haloes, const int64_t *offsets, const double *x,
                                    const double *y, const double *z, const double *vx, const double *vy,
                                    const double *vz, const double *m, const halma_unbind_params *params,
                                    uint8_t *bound, double *phi, double *halo_out, halma_stream_t stream) {
    if (!params) return fail(HALMA_ERR_INVALID, "params is NULL");
    const halma_unbind_params p = *params;
    if (n < 0 || n_haloes < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n >= (1ll << 31) - 64) return fail(HALMA_ERR_CAPACITY, "at most 2^31-65 particles per call");
    if (n_haloes >= (1ll << 31) - 1) return fail(HALMA_ERR_CAPACITY, "too many haloes");
    if (!(p.eps > 0.0) || !isfinite(p.eps)) return fail(HALMA_ERR_INVALID, "eps must be finite and > 0");
    if (!isfinite(p.G) || !isfinite(p.factor_v)) return fail(HALMA_ERR_INVALID, "G and factor_v must be finite");
    if (p.max_iter < 1 || p.max_iter > 1000) return fail(HALMA_ERR_INVALID, "max_iter must be in [1, 1000]");
    if (p.precision != HALMA_UNBIND_FP32C && p.precision != HALMA_UNBIND_FP64)
        return fail(HALMA_ERR_INVALID, "unknown precision %d", p.precision);
    if (!offsets || (n > 0 && (!x || !y || !z || !vx || !vy || !vz || !m || !bound)))
        return fail(HALMA_ERR_INVALID, "null pointer");
    if (n_haloes == 0) return HALMA_OK;
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    // the plan needs the offsets on the host
    std::vector<int64_t> h_off(n_haloes + 1);
    const bool dev_off = is_device_pointer(offsets);
    if (dev_off) {
        HALMA_CUDA(cudaMemcpyAsync(h_off.data(), offsets, sizeof(int64_t) * (n_haloes + 1), cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
    } else {
        memcpy(h_off.data(), offsets, sizeof(int64_t) * (n_haloes + 1));
    }
    if (h_off[0] != 0 || h_off[n_haloes] != n) return fail(HALMA_ERR_INVALID, "offsets must start at 0 and end at n");
    for (int64_t h = 0; h < n_haloes; ++h)
        if (h_off[h + 1] < h_off[h]) return fail(HALMA_ERR_INVALID, "offsets must be non-decreasing");
    Stager sg;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dvx = nullptr, *dvy = nullptr, *dvz = nullptr,
                 *dm = nullptr;
    unsigned char *db = nullptr;
    double *dphi = nullptr, *dout = nullptr;
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add(vx, n, true, false, &dvx);
    sg.add(vy, n, true, false, &dvy);
    sg.add(vz, n, true, false, &dvz);
    sg.add(m, n, true, false, &dm);
    sg.add((const unsigned char *)bound, n, false, true, &db);
    sg.add((const double *)phi, phi ? n : 0, false, true, &dphi);
    sg.add((const double *)halo_out, halo_out ? n_haloes * HALMA_UB_NFIELDS : 0, false, true, &dout);
    void *stage = nullptr;
    if (sg.any_host) {
        Layout L;
        sg.plan(L);
        HALMA_CUDA(cudaMallocAsync(&stage, L.total, st));
    }
    int s = sg.bind_and_upload(stage, st);
    if (s == HALMA_OK)
        s = unbind_device(n, (int)n_haloes, dev_off ? offsets : nullptr, h_off.data(), dx, dy, dz, dvx, dvy, dvz, dm,
                          p, db, dphi, dout, st);
    if (s == HALMA_OK) s = sg.download(st);
    if (stage) {
        cudaFreeAsync(stage, st);
        cudaStreamSynchronize(st);
    }
    return s;
}

extern "C" int halma_set_tile_table(int32_t n_classes, const int32_t *upper, const int32_t *t_per_class,
                                    int32_t slice_len) {
    if (n_classes < 1 || n_classes > kMaxTileClasses || !upper || !t_per_class)
        return fail(HALMA_ERR_INVALID, "tile table needs 1..%d classes", kMaxTileClasses);
    if (slice_len < 32 || slice_len % 32 != 0 || slice_len > (1 << 26))
        return fail(HALMA_ERR_INVALID, "source slice must be a positive multiple of 32 (at most 2^26)");
    TileTable t{};
    t.n = n_classes;
    t.slice = slice_len;
    for (int c = 0; c < n_classes; ++c) {
        const int v = t_per_class[c];
        if (v != 1 && v != 2 && v != 4) return fail(HALMA_ERR_INVALID, "tile shape must be 1, 2 or 4");
        if (upper[c] < 1 || (c > 0 && upper[c] <= upper[c - 1]))
            return fail(HALMA_ERR_INVALID, "class bounds must be positive and increasing");
        t.upper[c] = upper[c];
        t.t[c] = v;
    }
    std::lock_guard<std::mutex> guard(api_mutex());
    tile_table_ref() = t;
    return HALMA_OK;
}

extern "C" int halma_get_tile_table(int32_t *n_classes, int32_t *upper, int32_t *t_per_class,
                                    int32_t *slice_len) {
    if (!n_classes || !upper || !t_per_class || !slice_len) return fail(HALMA_ERR_INVALID, "null pointer");
    std::lock_guard<std::mutex> guard(api_mutex());
    const TileTable &t = tile_table_ref();
    *n_classes = t.n;
    *slice_len = t.slice;
    for (int c = 0; c < t.n; ++c) {
        upper[c] = t.upper[c];
        t_per_class[c] = t.t[c];
    }
    return HALMA_OK;
}
