// PCS + interlaced mass assignment with shared-memory tile accumulation
// (estimator.f:284-512, density mode; the same per-particle arithmetic as
// assign_pcs_kernel in mesh.cu).
//
// The direct kernel adds each of a particle's 2 x 64 weights straight into
// the grid with L2 atomics.  When there are many particles per cell the same
// cells are hit again and again; this form first bins the particles by the
// grid tile their stencil starts in, then lets one CTA per tile accumulate
// all of the tile's particles in shared memory and add the tile, halo
// included, to the grid once:
//
//   1. tile_bin_kernel    tile of each particle; per-tile counts (warp-
//                         aggregated atomics: lanes with the same tile add once)
//   2. tile_scan_kernel   exclusive scan of the counts (one CTA)
//   3. tile_fill_kernel   particle indices grouped by tile
//   4. tile_accum_kernel  per tile: shared-memory atomics into a (B+4)^3 x 2
//                         float block, then one global atomic per non-zero
//                         cell of the block
//
// Tiles: the grid is cut into B^3-cell tiles (the last tile along an axis
// may be shorter).  A particle with base cell m (per axis) touches cells
// m-2 .. m+2 of the two interlaced grids (m-2 .. m+1 of the standard grid,
// q-2 .. q+1 with q in {m, m+1} of the shifted one), so a particle whose
// first cell c = (m - 2) mod N lies in tile t touches only cells
// tB .. tB+B+3 (mod N): the block with its 4-cell halo.  Requires N >= B + 4.
#include "common.cuh"

namespace pyspec {

namespace asg {

constexpr int kThreads = 256;

__device__ __forceinline__ void pcs_w(float h, float* o) {
    const float h2 = __fmul_rn(h, h);
    const float om = __fsub_rn(1.0f, h);
    const float wm2 = __fmul_rn(__fmul_rn(om, om), om);
    const float wm1 = __fadd_rn(4.0f, __fmul_rn(__fsub_rn(__fmul_rn(3.0f, h), 6.0f), h2));
    const float wp2 = __fmul_rn(h2, h);
    const float wp1 = __fsub_rn(__fsub_rn(__fsub_rn(6.0f, wm2), wm1), wp2);
    o[0] = wm2; o[1] = wm1; o[2] = wp1; o[3] = wp2;
}

__device__ __forceinline__ int wrapi(int c, int n) {
    c %= n;
    return c < 0 ? c + n : c;
}

// base cell m of one coordinate (estimator.f:302, single precision, no FMA)
__device__ __forceinline__ int base_cell(float r, float kf_ks, float offset) {
    return __float2int_rz(__fadd_rn(__fadd_rn(__fmul_rn(kf_ks, r), 1.0f), offset));
}

struct Tiling {
    int n, B, nt1;      // grid size, tile edge, tiles per axis
    int64_t ntiles;
};

__device__ __forceinline__ int64_t tile_of(const float* __restrict__ xyz, int64_t np, int64_t i, float kf_ks,
                                           float offset, const Tiling& T) {
    int t[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) t[d] = wrapi(base_cell(xyz[d * np + i], kf_ks, offset) - 2, T.n) / T.B;
    return ((int64_t)t[2] * T.nt1 + t[1]) * T.nt1 + t[0];
}

__global__ void __launch_bounds__(kThreads) tile_bin_kernel(const float* __restrict__ xyz, int64_t np, float kf_ks,
                                                            float offset, Tiling T, int* __restrict__ tile,
                                                            int* __restrict__ count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool on = i < np;
    const int t = on ? (int)tile_of(xyz, np, i, kf_ks, offset, T) : -1;
    if (on) tile[i] = t;
    // lanes of the warp with the same tile add their number once
    const unsigned peers = __match_any_sync(0xffffffffu, t);
    const int leader = __ffs(peers) - 1;
    if (on && (threadIdx.x & 31) == leader) atomicAdd(count + t, __popc(peers));
}

// Exclusive scan of count[0..nt) into start[0..nt] (start[nt] = total) and a
// copy into cursor, by one CTA of 1024 threads (nt <= 2^24).
__global__ void __launch_bounds__(1024) tile_scan_kernel(const int* __restrict__ count, int64_t nt,
                                                         int* __restrict__ start, int* __restrict__ cursor) {
    __shared__ int part[1024];
    const int tid = threadIdx.x;
    const int64_t per = (nt + 1023) / 1024;
    const int64_t a = min(nt, tid * per), b = min(nt, a + per);
    int s = 0;
    for (int64_t k = a; k < b; ++k) s += count[k];
    part[tid] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {       // inclusive Hillis-Steele scan
        const int v = tid >= off ? part[tid - off] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    int run = part[tid] - s;                          // exclusive prefix of this segment
    for (int64_t k = a; k < b; ++k) {
        start[k] = run;
        cursor[k] = run;
        run += count[k];
    }
    if (tid == 1023) start[nt] = part[1023];
}

__global__ void __launch_bounds__(kThreads) tile_fill_kernel(const int* __restrict__ tile, int64_t np,
                                                             int* __restrict__ cursor, int* __restrict__ order) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool on = i < np;
    const int t = on ? tile[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, t);
    const int leader = __ffs(peers) - 1;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (on && lane == leader) base = atomicAdd(cursor + t, __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (on) order[base + __popc(peers & ((1u << lane) - 1u))] = (int)i;
}

// One CTA per tile: the tile's particles into a shared (B+4)^3 block of
// (standard, interlaced) float pairs, then the block into the grid.
template <int B>
__global__ void __launch_bounds__(kThreads) tile_accum_kernel(const float* __restrict__ xyz,
                                                              const float* __restrict__ w, int64_t np, float kf_ks,
                                                              float offset, Tiling T, const int* __restrict__ start,
                                                              const int* __restrict__ order,
                                                              float* __restrict__ grid) {
    constexpr int E = B + 4;
    extern __shared__ float2 blk[];                   // E^3 (standard, interlaced) pairs
    const int64_t t = blockIdx.x;
    const int p0 = start[t], p1 = start[t + 1];
    if (p0 == p1) return;                              // CTA-uniform
    const int n = T.n;
    const int tx = (int)(t % T.nt1), ty = (int)((t / T.nt1) % T.nt1), tz = (int)(t / ((int64_t)T.nt1 * T.nt1));
    const int ox = tx * B, oy = ty * B, oz = tz * B;   // first cell of the block (before wrap)
    for (int k = threadIdx.x; k < E * E * E; k += blockDim.x) blk[k] = make_float2(0.f, 0.f);
    __syncthreads();
    const int o[3] = {ox, oy, oz};
    if ((p1 - p0) * 8 > 4 * (int)blockDim.x) {
        // dense tile: one thread per particle, both grids and all 64 cells
        for (int k = p0 + threadIdx.x; k < p1; k += blockDim.x) {
            const int64_t i = order[k];
            const float we = w ? w[i] : 1.0f;
            int base[2][3];
            float wt[2][3][4];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float r = xyz[d * np + i];
                const float rx = __fadd_rn(__fadd_rn(__fmul_rn(kf_ks, r), 1.0f), offset);   // estimator.f:302
                const float tq = __fadd_rn(rx, 0.5f);                                      // estimator.f:305
                const int m = __float2int_rz(rx);
                const int q = __float2int_rz(tq);
                pcs_w(__fsub_rn(rx, (float)m), wt[0][d]);
                pcs_w(__fsub_rn(tq, (float)q), wt[1][d]);
                base[0][d] = m;
                base[1][d] = q;
            }
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                int lc[3][4];                            // block-local cells per axis, in [0, E)
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int c = 0; c < 4; ++c) lc[d][c] = wrapi(base[s][d] - 2 + c - o[d], n);
#pragma unroll
                for (int c3 = 0; c3 < 4; ++c3)
#pragma unroll
                    for (int c2 = 0; c2 < 4; ++c2) {
                        float* row = reinterpret_cast<float*>(blk + (lc[2][c3] * E + lc[1][c2]) * E) + s;
#pragma unroll
                        for (int c1 = 0; c1 < 4; ++c1) {
                            // estimator.f:380: ((hx*hy)*hz)*we
                            const float v = __fmul_rn(__fmul_rn(__fmul_rn(wt[s][0][c1], wt[s][1][c2]), wt[s][2][c3]), we);
                            atomicAdd(row + 2 * lc[0][c1], v);
                        }
                    }
            }
        }
    } else {
    // sparse tile: eight work items per particle, (grid s, z offset c3), each
    // adding its 4 x 4 weights (short atomic chains, and the CTA's threads
    // stay busy when the tile holds fewer particles than threads)
    for (int it = threadIdx.x; it < (p1 - p0) * 8; it += blockDim.x) {
        const int64_t i = order[p0 + (it >> 3)];
        const int s = (it >> 2) & 1, c3 = it & 3;
        const float we = w ? w[i] : 1.0f;
        int base[3];
        float wt[3][4];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float r = xyz[d * np + i];
            const float rx = __fadd_rn(__fadd_rn(__fmul_rn(kf_ks, r), 1.0f), offset);   // estimator.f:302
            const float tq = s ? __fadd_rn(rx, 0.5f) : rx;                             // estimator.f:305
            const int m = __float2int_rz(tq);
            pcs_w(__fsub_rn(tq, (float)m), wt[d]);
            base[d] = m;
        }
        int lc[2][4];                                // block-local cells along x and y, in [0, E)
#pragma unroll
        for (int d = 0; d < 2; ++d)
#pragma unroll
            for (int c = 0; c < 4; ++c) lc[d][c] = wrapi(base[d] - 2 + c - o[d], n);
        const int lz = wrapi(base[2] - 2 + c3 - o[2], n);
#pragma unroll
        for (int c2 = 0; c2 < 4; ++c2) {
            float* row = reinterpret_cast<float*>(blk + (lz * E + lc[1][c2]) * E) + s;
#pragma unroll
            for (int c1 = 0; c1 < 4; ++c1) {
                // estimator.f:380: ((hx*hy)*hz)*we
                const float v = __fmul_rn(__fmul_rn(__fmul_rn(wt[0][c1], wt[1][c2]), wt[2][c3]), we);
                atomicAdd(row + 2 * lc[0][c1], v);
            }
        }
    }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < E * E * E; k += blockDim.x) {
        const float2 v = blk[k];
        if (v.x == 0.f && v.y == 0.f) continue;
        const int lx = k % E, ly = (k / E) % E, lz = k / (E * E);
        const int gx = wrapi(ox + lx, n), gy = wrapi(oy + ly, n), gz = wrapi(oz + lz, n);
        float* g = grid + 2 * (((int64_t)gz * n + gy) * n + gx);
        // both grids of the cell with one 8-byte vector reduction
        asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" :: "l"(g), "f"(v.x), "f"(v.y) : "memory");
    }
}

inline size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

inline Tiling tiling(int n, int B) {
    Tiling T;
    T.n = n;
    T.B = B;
    T.nt1 = (n + B - 1) / B;
    T.ntiles = (int64_t)T.nt1 * T.nt1 * T.nt1;
    return T;
}

}  // namespace asg
}  // namespace pyspec

using namespace pyspec;

extern "C" size_t pyspec_assign_tiled_workspace(int64_t np, int ngrid, int tile) {
    if (np < 0 || ngrid < 1 || (tile != 4 && tile != 8 && tile != 16)) return 0;
    const asg::Tiling T = asg::tiling(ngrid, tile);
    const size_t nt = (size_t)T.ntiles;
    return asg::al256(nt * 4) + asg::al256((nt + 1) * 4) + asg::al256(nt * 4) + 2 * asg::al256((size_t)np * 4) + 256;
}

extern "C" int pyspec_assign_pcs_interlaced_tiled(const float* xyz, const float* w, int64_t np, int ngrid,
                                                  float kf_ks, float offset, int tile, float* grid,
                                                  void* workspace, size_t ws_bytes, void* stream) {
    PYSPEC_CHECK_ARG(np >= 0, "np < 0");
    PYSPEC_CHECK_ARG(tile == 4 || tile == 8 || tile == 16, "tile=%d must be 4, 8 or 16", tile);
    PYSPEC_CHECK_ARG(ngrid >= tile + 4, "ngrid=%d too small for tile %d (needs ngrid >= tile + 4)", ngrid, tile);
    PYSPEC_CHECK_ARG(np < (int64_t)1 << 31, "np=%lld exceeds the int32 particle index", (long long)np);
    if (np == 0) return PYSPEC_OK;
    PYSPEC_CHECK_ARG(xyz && grid && workspace, "NULL pointer");
    const size_t need = pyspec_assign_tiled_workspace(np, ngrid, tile);
    if (ws_bytes < need) {
        set_error("assignment workspace %zu bytes < required %zu", ws_bytes, need);
        return PYSPEC_E_WORKSPACE;
    }
    const asg::Tiling T = asg::tiling(ngrid, tile);
    PYSPEC_CHECK_ARG(T.ntiles < ((int64_t)1 << 24), "too many tiles (%lld)", (long long)T.ntiles);
    const size_t nt = (size_t)T.ntiles;
    char* p = reinterpret_cast<char*>(workspace);
    int* count = reinterpret_cast<int*>(p);
    p += asg::al256(nt * 4);
    int* start = reinterpret_cast<int*>(p);
    p += asg::al256((nt + 1) * 4);
    int* cursor = reinterpret_cast<int*>(p);
    p += asg::al256(nt * 4);
    int* tid = reinterpret_cast<int*>(p);
    p += asg::al256((size_t)np * 4);
    int* order = reinterpret_cast<int*>(p);
    cudaStream_t st = as_stream(stream);
    PYSPEC_CUDA(cudaMemsetAsync(count, 0, nt * 4, st));
    const unsigned nb = (unsigned)((np + asg::kThreads - 1) / asg::kThreads);
    asg::tile_bin_kernel<<<nb, asg::kThreads, 0, st>>>(xyz, np, kf_ks, offset, T, tid, count);
    PYSPEC_LAUNCH_CHECK();
    asg::tile_scan_kernel<<<1, 1024, 0, st>>>(count, T.ntiles, start, cursor);
    PYSPEC_LAUNCH_CHECK();
    asg::tile_fill_kernel<<<nb, asg::kThreads, 0, st>>>(tid, np, cursor, order);
    PYSPEC_LAUNCH_CHECK();
#define PYSPEC_TILE_ACCUM(BV)                                                                              \
    do {                                                                                                   \
        const size_t sm = sizeof(float2) * (BV + 4) * (BV + 4) * (BV + 4);                                 \
        PYSPEC_TRY(allow_smem((const void*)asg::tile_accum_kernel<BV>, sm));                               \
        asg::tile_accum_kernel<BV><<<(unsigned)T.ntiles, asg::kThreads, sm, st>>>(xyz, w, np, kf_ks, offset, T, \
                                                                               start, order, grid);        \
    } while (0)
    switch (tile) {
        case 4: PYSPEC_TILE_ACCUM(4); break;
        case 8: PYSPEC_TILE_ACCUM(8); break;
        default: PYSPEC_TILE_ACCUM(16); break;
    }
#undef PYSPEC_TILE_ACCUM
    PYSPEC_LAUNCH_CHECK();
    count_launch(4);
    return PYSPEC_OK;
}
