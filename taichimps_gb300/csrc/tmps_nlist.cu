// Neighbor build and contact-history carry-over (FP64, exact).
//
// Atoms are binned in lamda coordinates exactly as NeighborList.get_cell_coord
// does (neighbor.py:191-206), then physically re-sorted: cells laid out along a
// Morton curve, atoms inside a cell by insertion index.  The full list (both
// i->j and j->i) is then built from the 27-cell stencil with the reference's
// periodic-wrap and single-bin skip rules (neighbor.py:329-351) and the exact
// FP64 cut test (ri + rj + skin)^2 (neighbor.py:355-359), so the pair set is
// bit-identical to the reference's half list on the same positions.
#include <mutex>

#include "tmps_common.cuh"

using namespace tmps;

namespace {

constexpr int kBlock = 256;
constexpr int kScanBlock = 1024;

// Cell of one position: floor(((x - lo) / prd) / csize), clamped.  The
// reference's lamda for an orthogonal box adds products with zero tilt terms,
// which leave the quotient unchanged.
//
// Only the floor of the quotient t matters.  An FP32 estimate of t from the
// truncated position (approx_f32: integer operations) is within 4e-6 of
// ((|x| + |lo|) / h + |t| + 1) of the exact chain's quotient (h = prd csize,
// the cell edge; the bound is four times the truncation and FP32 rounding
// errors), so wherever the estimate lies further than that from an integer
// both floors agree; within it (a few atoms in 10^4, or a NaN) the exact
// chain of two correctly rounded FP64 divisions decides.  No FP64 arithmetic
// otherwise: this part's FP64 pipe is narrow.
struct AxisBin {
    double lo, prd, csize;
    float lo32, rprd32, rcs32, rh32;  // FP32 lo, 1/prd, 1/csize, 1/(prd csize)
    int g;
};

__device__ __forceinline__ int cell_axis(double x, const AxisBin& ax) {
    const float xf = approx_f32(x);
    const float t = ((xf - ax.lo32) * ax.rprd32) * ax.rcs32;
    const float qf = floorf(t);
    const float r = t - qf;
    const float m = 4e-6f * (((fabsf(xf) + fabsf(ax.lo32)) * ax.rh32 + fabsf(t)) + 1.0f);
    if (r > m && r < 1.0f - m)
        return qf >= (float)(ax.g - 1) ? ax.g - 1 : (qf > 0.0f ? (int)qf : 0);
    const double q = floor(__ddiv_rn(__ddiv_rn(__dsub_rn(x, ax.lo), ax.prd), ax.csize));
    // clamp in floating point first so a stray NaN/Inf cannot overflow the
    // int conversion; NaN falls to cell 0
    return q >= (double)(ax.g - 1) ? ax.g - 1 : (q > 0.0 ? (int)q : 0);
}

__global__ void __launch_bounds__(kBlock) k_bin(tmps_atoms a, const tmps_box* __restrict__ b,
                                                const int32_t* __restrict__ rank, int32_t* old_cell,
                                                int32_t* count, int32_t* status) {
    __shared__ AxisBin sax[3];
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        AxisBin ax;
        ax.lo = b->lo[k];
        ax.prd = b->prd[k];
        ax.csize = b->csize[k];
        ax.g = b->g[k];
        ax.lo32 = approx_f32(ax.lo);
        ax.rprd32 = (float)(1.0 / ax.prd);
        ax.rcs32 = (float)(1.0 / ax.csize);
        ax.rh32 = (float)(1.0 / (ax.prd * ax.csize));
        sax[k] = ax;
    }
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double4 x = ld4(a.xr, i);
    if (!finite_bits(x.x) || !finite_bits(x.y) || !finite_bits(x.z)) atomicOr(status, TMPS_STATUS_NONFINITE);
    const int cx = cell_axis(x.x, sax[0]), cy = cell_axis(x.y, sax[1]), cz = cell_axis(x.z, sax[2]);
    int lin = cx + cy * sax[0].g + cz * sax[0].g * sax[1].g;
    old_cell[i] = lin;
    atomicAdd(&count[rank[lin]], 1);
}

// Exclusive scan of `count` (length m, by Morton rank) into start[0..m],
// start[m] the total.  Two launches over tiles of kScanTile cells, one block
// of kScanBlock threads per tile (each thread four consecutive cells):
// k_scan_tiles writes each tile's total to tile_sum[tile]; k_scan_apply
// adds the totals of the earlier tiles to a block-wide scan of its own tile.
// Runs once per rebuild; ~74k cells (the 1M-sphere grid) are 19 tiles.
constexpr int kScanTile = 4 * kScanBlock;

__device__ __forceinline__ int32_t scan_tile_block(int32_t v, int32_t* wsum, int32_t& total) {
    // exclusive block scan of one value per thread; total of the block
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t s = wsum[lane];  // kScanBlock / 32 == 32 warps
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        wsum[lane] = s;
    }
    __syncthreads();
    total = wsum[31];
    return (w > 0 ? wsum[w - 1] : 0) + x - v;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_tiles(const int32_t* __restrict__ count, int m,
                                                          int32_t* __restrict__ tile_sum) {
    __shared__ int32_t wsum[kScanBlock / 32];
    const int c0 = blockIdx.x * kScanTile + 4 * threadIdx.x;
    int32_t v = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (c0 + k < m) v += count[c0 + k];
    int32_t total;
    scan_tile_block(v, wsum, total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_apply(const int32_t* __restrict__ count,
                                                          int32_t* __restrict__ start, int m,
                                                          const int32_t* __restrict__ tile_sum) {
    __shared__ int32_t wsum[kScanBlock / 32];
    __shared__ int32_t base;
    if (threadIdx.x < 32) {
        int32_t s = 0;
        for (int t = threadIdx.x; t < (int)blockIdx.x; t += 32) s += tile_sum[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) base = s;
    }
    const int c0 = blockIdx.x * kScanTile + 4 * threadIdx.x;
    int32_t cnt[4], v = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        cnt[k] = c0 + k < m ? count[c0 + k] : 0;
        v += cnt[k];
    }
    int32_t total;
    int32_t run = scan_tile_block(v, wsum, total) + base;  // scan_tile_block's barriers publish `base`
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (c0 + k < m) start[c0 + k] = run;
        run += cnt[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) start[m] = base + total;
}

__global__ void __launch_bounds__(kBlock) k_scatter(int n, const int32_t* __restrict__ rank,
                                                    const int32_t* __restrict__ old_cell,
                                                    const int32_t* __restrict__ start, int32_t* fill,
                                                    int32_t* order) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int r = rank[old_cell[i]];
    int slot = atomicAdd(&fill[r], 1);
    order[start[r] + slot] = i;
}

// Within each cell, order atoms by insertion index: the layout then depends
// only on positions, not on which atomics won the scatter.
__global__ void __launch_bounds__(kBlock) k_cell_sort(int m, const int32_t* __restrict__ start,
                                                      const int32_t* __restrict__ uid, int32_t* order) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    int beg = start[r], end = start[r + 1];
    for (int p = beg + 1; p < end; ++p) {
        int v = order[p];
        int key = uid[v];
        int q = p - 1;
        while (q >= beg && uid[order[q]] > key) {
            order[q + 1] = order[q];
            --q;
        }
        order[q + 1] = v;
    }
}

// Gather every per-atom array into the new order; store x0 for the skin check
// and, when `off32` is given, each position as an FP32 offset from the origin
// lo + c h of its own cell (h = prd / g), radius in .w, for the build's
// prefilter.
__global__ void __launch_bounds__(kBlock) k_permute(tmps_atoms src, tmps_atoms dst,
                                                    const tmps_box* __restrict__ b,
                                                    const int32_t* __restrict__ order,
                                                    const int32_t* __restrict__ old_cell,
                                                    int32_t* cell_of, float4* __restrict__ off32) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = src.n;
    if (p >= n) return;
    int i = order[p];
    double4 x = ld4(src.xr, i);
    if (off32) {
        const int gx = b->g[0], gxy = b->g[0] * b->g[1];
        const int lin = old_cell[i];
        const int cz = lin / gxy, cy = (lin - cz * gxy) / gx, cx = lin - cz * gxy - cy * gx;
        const int cc[3] = {cx, cy, cz};
        const double xx[3] = {x.x, x.y, x.z};
        float o[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double h = b->hcell[k];  // prd / g, kept with the box (no division per atom)
            o[k] = f32_rn(xx[k] - (b->lo[k] + (double)cc[k] * h));
        }
        off32[p] = make_float4(o[0], o[1], o[2], f32_rn(x.w));
    }
    st4(dst.xr, p, x);
    st4(dst.vm, p, ld4(src.vm, i));
    st4(dst.om, p, ld4(src.om, i));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        dst.f[k * n + p] = src.f[k * n + i];
        dst.torque[k * n + p] = src.torque[k * n + i];
    }
    if (src.virial && dst.virial) {
#pragma unroll
        for (int k = 0; k < 6; ++k) dst.virial[k * n + p] = src.virial[k * n + i];
    }
    dst.tag[p] = src.tag[i];
    dst.uid[p] = src.uid[i];
    dst.x0[p] = x.x;
    dst.x0[n + p] = x.y;
    dst.x0[2 * n + p] = x.z;
    cell_of[p] = old_cell[i];
}

// The three cells of one axis at stencil offsets -1, 0, +1 (neighbor.py:
// 329-351): wrapped on a periodic axis (a stencil offset is at most one cell,
// so one add or subtract does it), -1 where the stencil leaves a non-periodic
// grid, and -1 for the off-centre cells of a periodic axis of a single bin.
struct AxisCells {
    int m, c, p;  // offsets -1, 0, +1
    __device__ __forceinline__ int at(int o) const { return o < 0 ? m : (o == 0 ? c : p); }
};

__device__ __forceinline__ AxisCells axis_cells(int c, int g, int per) {
    AxisCells a;
    a.c = c;
    if (per == 1) {
        a.m = g == 1 ? -1 : (c == 0 ? g - 1 : c - 1);
        a.p = g == 1 ? -1 : (c == g - 1 ? 0 : c + 1);
    } else {
        a.m = c > 0 ? c - 1 : -1;
        a.p = c < g - 1 ? c + 1 : -1;
    }
    return a;
}

// The full list.  Stencil order and wrap/skip rules of neighbor.py:329-351;
// the cut test is done with explicit round-to-nearest operations so no
// multiply-add contraction can move a pair across the cut.
//
// With `off32` (and every periodic dimension at least 3 cells wide) each
// candidate first meets an FP32 test on cell-local offsets: a pair within
// the cut lies in adjacent cells, so its separation is exactly
// (o_i - o_j) - offset * h, which FP32 carries to ~1e-6 of (h + |o|).  A
// candidate is dropped when its FP32 distance exceeds the cut by more than
// ten times that error bound, and taken when it falls short of the cut by
// as much (the cut is at most one cell, under a third of the box, so the
// minimum image the FP64 test would pick is the stencil's image); only the
// candidates in that narrow band get the exact FP64 test.  The list is the
// pair set the FP64 test alone gives, at a sliver of the FP64 work (this
// part's FP64 pipe is ~70x narrower than its FP32 pipe, and the exact test
// divides).
__global__ void __launch_bounds__(kBlock) k_build(tmps_atoms a, const tmps_box* __restrict__ b,
                                                  double skin, const int32_t* __restrict__ cell_of,
                                                  const int32_t* __restrict__ rank,
                                                  const int32_t* __restrict__ start, tmps_nlist nl,
                                                  const float4* __restrict__ off32, int32_t* status) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.n;
    if (p >= n) return;
    const int gx = b->g[0], gy = b->g[1], gz = b->g[2], gxy = gx * gy;
    const int px = b->per[0], py = b->per[1], pz = b->per[2];
    const int lin = cell_of[p];
    const int cz = lin / gxy, cy = (lin - cz * gxy) / gx, cx = lin - cz * gxy - cy * gx;
    const AxisCells nxs = axis_cells(cx, gx, px), nys = axis_cells(cy, gy, py), nzs = axis_cells(cz, gz, pz);
    const double4 xi = ld4(a.xr, p);
    const double prd[3] = {b->prd[0], b->prd[1], b->prd[2]};
    const bool pre = off32 != nullptr && !(px == 1 && gx < 3) && !(py == 1 && gy < 3) && !(pz == 1 && gz < 3);
    float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
    float h32[3] = {0.f, 0.f, 0.f}, base = 0.f, wi = 0.f;
    const float skin32 = (float)skin;
    if (pre) {
        oi = off32[p];
        float hsum = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            h32[k] = f32_rn(b->hcell[k]);  // hcell = prd / g, the box keeps it so
            hsum += h32[k];
        }
        base = hsum + fmaxf(fmaxf(fabsf(oi.x), fabsf(oi.y)), fabsf(oi.z));
        wi = oi.w + skin32;
    }
    int count = 0;
    bool overflow = false;
    for (int ox = -1; ox <= 1; ++ox) {
        const int nx = nxs.at(ox);
        if (nx < 0) continue;
        for (int oy = -1; oy <= 1; ++oy) {
            const int ny = nys.at(oy);
            if (ny < 0) continue;
            for (int oz = -1; oz <= 1; ++oz) {
                const int nz = nzs.at(oz);
                if (nz < 0) continue;
                const int r = rank[nx + ny * gx + nz * gxy];
                const int code = (ox + 1) + 3 * (oy + 1) + 9 * (oz + 1);
                const int beg = start[r], end = start[r + 1];
                // the row atom's offset moved by the stencil offset: d = (o_i - f) - o_j
                const float ax = oi.x - (float)ox * h32[0], ay = oi.y - (float)oy * h32[1],
                            az = oi.z - (float)oz * h32[2];
                for (int q = beg; q < end; ++q) {
                    if (q == p) continue;
                    bool inside = false;
                    if (pre) {
                        // within reach beyond doubt, out of reach beyond doubt, or the
                        // exact test: the slack is ten times the FP32 error bound of
                        // d and of the cut, ~1e-6 of the magnitudes involved
                        const float4 oj = off32[q];
                        const float dx = ax - oj.x, dy = ay - oj.y, dz = az - oj.z;
                        const float rq = (dx * dx + dy * dy) + dz * dz;
                        const float mj = fmaxf(fmaxf(fabsf(oj.x), fabsf(oj.y)), fabsf(oj.z));
                        const float cut = wi + oj.w;
                        const float slack = 1e-5f * ((base + mj) + cut);
                        const float lim = cut + slack, near = cut - slack;
                        if (!(rq < lim * lim) && rq == rq) continue;  // a NaN goes on to the exact test
                        inside = near > 0.0f && rq < near * near;
                    }
                    if (inside) {
                        if (count < nl.slots) {
                            nl.nbr[(size_t)count * n + p] = q | (code << kNbrIndexBits);
                            ++count;
                        } else {
                            overflow = true;
                        }
                        continue;
                    }
                    const double4 xj = ld4(a.xr, q);
                    double d[3] = {__dsub_rn(xi.x, xj.x), __dsub_rn(xi.y, xj.y), __dsub_rn(xi.z, xj.z)};
#pragma unroll
                    for (int k = 0; k < 3; ++k)
                        if (b->per[k] == 1)
                            d[k] = __dsub_rn(d[k], __dmul_rn(prd[k], round(__ddiv_rn(d[k], prd[k]))));
                    double rsq = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])),
                                           __dmul_rn(d[2], d[2]));
                    double rad = __dadd_rn(__dadd_rn(xi.w, xj.w), skin);
                    if (rsq < __dmul_rn(rad, rad)) {
                        if (count < nl.slots) {
                            nl.nbr[(size_t)count * n + p] = q | (code << kNbrIndexBits);
                            ++count;
                        } else {
                            overflow = true;
                        }
                    }
                }
            }
        }
    }
    nl.nnb[p] = count;
    if (overflow) atomicOr(status, TMPS_STATUS_NLIST_OVERFLOW);
}

// ContactHistory save/restore (contact_history.py:91-139) in one pass: for
// each slot of the new list, find the same partner among the old row's
// touching slots and carry its shear (and rolling displacement, when both
// lists hold one) over; anything else starts at zero.
__global__ void __launch_bounds__(kBlock) k_history_remap(tmps_nlist o, tmps_nlist nw,
                                                          const int32_t* __restrict__ order) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = nw.n;
    if (p >= n) return;
    const int po = order[p];
    const uint64_t otouch = o.touch[po];
    const int onn = o.nnb[po];
    const int nn = nw.nnb[p];
    uint64_t bits = 0;
    const bool roll = o.rolling != nullptr && nw.rolling != nullptr;
    for (int k = 0; k < nn; ++k) {
        const int qo = order[nw.nbr[(size_t)k * n + p] & kNbrIndexMask];
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, r0 = 0.0, r1 = 0.0, r2 = 0.0;
        if (otouch) {
            for (int ko = 0; ko < onn; ++ko) {
                if (!((otouch >> ko) & 1ull)) continue;
                if ((o.nbr[(size_t)ko * n + po] & kNbrIndexMask) != qo) continue;
                const size_t ss = (size_t)o.slots * n;
                s0 = o.shear[(size_t)ko * n + po];
                s1 = o.shear[ss + (size_t)ko * n + po];
                s2 = o.shear[2 * ss + (size_t)ko * n + po];
                if (roll) {
                    r0 = o.rolling[(size_t)ko * n + po];
                    r1 = o.rolling[ss + (size_t)ko * n + po];
                    r2 = o.rolling[2 * ss + (size_t)ko * n + po];
                }
                bits |= 1ull << k;
                break;
            }
        }
        const size_t ns = (size_t)nw.slots * n;
        nw.shear[(size_t)k * n + p] = s0;
        nw.shear[ns + (size_t)k * n + p] = s1;
        nw.shear[2 * ns + (size_t)k * n + p] = s2;
        if (roll) {
            nw.rolling[(size_t)k * n + p] = r0;
            nw.rolling[ns + (size_t)k * n + p] = r1;
            nw.rolling[2 * ns + (size_t)k * n + p] = r2;
        }
    }
    nw.touch[p] = bits;
}

bool launch_ok() { return cudaPeekAtLastError() == cudaSuccess; }

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// start = exclusive scan of count over m cells; tile_sum (at least one word per
// kScanTile cells, m words always suffice) holds the tile totals in between
void scan_cells(const int32_t* count, int32_t* start, int32_t* tile_sum, int m, cudaStream_t s) {
    const int tiles = (m + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<tiles, kScanBlock, 0, s>>>(count, m, tile_sum);
    k_scan_apply<<<tiles, kScanBlock, 0, s>>>(count, start, m, tile_sum);
}

}  // namespace

extern "C" {

int64_t tmps_nlist_workspace_bytes(int32_t n, int32_t ncell) {
    if (n < 0 || ncell < 0) return -1;
    // count[ncell], start[ncell+1], fill[ncell], old_cell[n], off32[n]
    return (int64_t)(align256((size_t)ncell * 4) + align256((size_t)(ncell + 1) * 4) +
                     align256((size_t)ncell * 4) + align256((size_t)n * 4) + align256((size_t)n * 16));
}

int tmps_nlist_build(const tmps_atoms* src, const tmps_atoms* dst, const tmps_box* d_box,
                     int32_t ncell, double skin, const int32_t* cell_rank, int32_t* order,
                     int32_t* cell_of, const tmps_nlist* nl, void* workspace,
                     int64_t workspace_bytes, int32_t* d_status, void* stream) {
    if (!src || !dst || !d_box || !cell_rank || !order || !cell_of || !nl || !workspace || !d_status)
        return TMPS_ERR_BAD_ARG;
    const int n = src->n;
    if (n < 0 || dst->n != n || nl->n != n || nl->slots < 1 || nl->slots > kMaxSlots ||
        n > kNbrIndexMask || !dst->x0)
        return TMPS_ERR_BAD_ARG;
    if (n == 0) return TMPS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int m = ncell;
    if (m < 1 || workspace_bytes < tmps_nlist_workspace_bytes(n, m)) return TMPS_ERR_BAD_ARG;
    char* w = (char*)workspace;
    int32_t* count = (int32_t*)w;
    w += align256((size_t)m * 4);
    int32_t* start = (int32_t*)w;
    w += align256((size_t)(m + 1) * 4);
    int32_t* fill = (int32_t*)w;
    w += align256((size_t)m * 4);
    int32_t* old_cell = (int32_t*)w;
    w += align256((size_t)n * 4);
    float4* off32 = (float4*)w;

    if (cudaMemsetAsync(count, 0, (size_t)m * 4, s) != cudaSuccess) return TMPS_ERR_CUDA;
    const int gb = grid_for(n, kBlock);
    k_bin<<<gb, kBlock, 0, s>>>(*src, d_box, cell_rank, old_cell, count, d_status);
    scan_cells(count, start, fill, m, s);
    // `fill` held the scan's tile totals; the scatter counts in it from zero
    if (cudaMemsetAsync(fill, 0, (size_t)m * 4, s) != cudaSuccess) return TMPS_ERR_CUDA;
    k_scatter<<<gb, kBlock, 0, s>>>(n, cell_rank, old_cell, start, fill, order);
    k_cell_sort<<<grid_for(m, kBlock), kBlock, 0, s>>>(m, start, src->uid, order);
    k_permute<<<gb, kBlock, 0, s>>>(*src, *dst, d_box, order, old_cell, cell_of, off32);
    k_build<<<gb, kBlock, 0, s>>>(*dst, d_box, skin, cell_of, cell_rank, start, *nl, off32, d_status);
    note_launches(7);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_history_remap(const tmps_nlist* old_nl, const tmps_nlist* new_nl, const int32_t* order,
                       void* stream) {
    if (!old_nl || !new_nl || !order || old_nl->n != new_nl->n) return TMPS_ERR_BAD_ARG;
    if (new_nl->n == 0) return TMPS_OK;
    k_history_remap<<<grid_for(new_nl->n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(*old_nl, *new_nl,
                                                                                     order);
    note_launches(1);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Neighbor build without any allocation by anyone.
//
// tmps_nlist_build wants a scratch buffer from the caller.  Some callers have
// no way to provide one: a host whose device memory all belongs to its own
// fixed arena, code that runs while a CUDA graph is being captured (where
// cudaMalloc is not allowed), or a foreign-language host that can only hand
// over the particle arrays it registered.  For them the scratch lives here, in
// one static device array of fixed size that every GPU which loads this
// library keeps until the process exits.  Its limits are stated in the header
// (TMPS_NOALLOC_MAX_ATOMS, TMPS_NOALLOC_MAX_CELLS).
namespace {

constexpr size_t kWords(size_t b) { return (b + 255) / 256 * 64; }  // 256-byte aligned, in int32 words
constexpr size_t kCountWords = kWords((size_t)TMPS_NOALLOC_MAX_CELLS * 4);
constexpr size_t kStartWords = kWords(((size_t)TMPS_NOALLOC_MAX_CELLS + 1) * 4);
constexpr size_t kFillWords = kWords((size_t)TMPS_NOALLOC_MAX_CELLS * 4);
constexpr size_t kCellWords = kWords((size_t)TMPS_NOALLOC_MAX_ATOMS * 4);
constexpr size_t kOffWords = kWords((size_t)TMPS_NOALLOC_MAX_ATOMS * 16);  // float4 cell-local offsets
constexpr size_t kScratchWords = kCountWords + kStartWords + kFillWords + kCellWords + kOffWords;

static __device__ __align__(256) int32_t g_build_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
int32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_build_scratch on the current device, looked up once per
// device (the host-side name is only a stand-in, not a device address).
int32_t* scratch_on_current_device() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_build_scratch) != cudaSuccess) return nullptr;
        g_scratch_ptr[dev] = static_cast<int32_t*>(p);
    }
    return g_scratch_ptr[dev];
}

}  // namespace

extern "C" int tmps_nlist_build_noalloc(const tmps_atoms* src, const tmps_atoms* dst, const tmps_box* d_box,
                                        int32_t ncell, double skin, const int32_t* cell_rank, int32_t* order,
                                        int32_t* cell_of, const tmps_nlist* nl, int32_t* d_status,
                                        void* stream) {
    if (!src || !dst || !d_box || !cell_rank || !order || !cell_of || !nl || !d_status) return TMPS_ERR_BAD_ARG;
    const int n = src->n;
    if (n < 0 || dst->n != n || nl->n != n || nl->slots < 1 || nl->slots > kMaxSlots || !dst->x0 || ncell < 1)
        return TMPS_ERR_BAD_ARG;
    if (n > TMPS_NOALLOC_MAX_ATOMS || ncell > TMPS_NOALLOC_MAX_CELLS) return TMPS_ERR_TOO_LARGE;
    if (n == 0) return TMPS_OK;
    int32_t* base = scratch_on_current_device();
    if (!base) return TMPS_ERR_CUDA;
    int32_t* count = base;
    int32_t* start = count + kCountWords;
    int32_t* fill = start + kStartWords;
    int32_t* old_cell = fill + kFillWords;
    float4* off32 = reinterpret_cast<float4*>(old_cell + kCellWords);  // 256-byte aligned
    cudaStream_t s = (cudaStream_t)stream;
    const int m = ncell;
    // the previous call left its counts behind: both counters must start at zero
    if (cudaMemsetAsync(count, 0, (size_t)m * 4, s) != cudaSuccess) return TMPS_ERR_CUDA;
    const int gb = grid_for(n, kBlock);
    k_bin<<<gb, kBlock, 0, s>>>(*src, d_box, cell_rank, old_cell, count, d_status);
    scan_cells(count, start, fill, m, s);
    // `fill` held the scan's tile totals; the scatter counts in it from zero
    if (cudaMemsetAsync(fill, 0, (size_t)m * 4, s) != cudaSuccess) return TMPS_ERR_CUDA;
    k_scatter<<<gb, kBlock, 0, s>>>(n, cell_rank, old_cell, start, fill, order);
    k_cell_sort<<<grid_for(m, kBlock), kBlock, 0, s>>>(m, start, src->uid, order);
    k_permute<<<gb, kBlock, 0, s>>>(*src, *dst, d_box, order, old_cell, cell_of, off32);
    k_build<<<gb, kBlock, 0, s>>>(*dst, d_box, skin, cell_of, cell_rank, start, *nl, off32, d_status);
    note_launches(7);
    return launch_ok() ? TMPS_OK : TMPS_ERR_CUDA;
}
