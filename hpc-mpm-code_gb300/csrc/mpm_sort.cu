// Particle binning and sorting.
//
// MeshPointLinklist (module/material_point.cpp:52-78) rebuilds a per-cell
// linked list every step; here every kernel recomputes a particle's cell from
// its position (the per-step binning), and every resort_period steps the
// particles are physically reordered by
//     (4x4x8-cell brick, cell inside the brick, load index)
// so that one CTA owns a brick and one thread owns a cell.  The order inside
// a cell is the load order (the reference visits a cell's particles in index
// order too), which makes the reordering deterministic.
//
//   k_bin         brick key + brick histogram
//   k_scan_up / k_scan_mid / k_scan_down
//                 brick starts, work-item list (chunks of <= CHUNK particles),
//                 list of non-empty bricks: a three-launch scan over segments
//   k_scatter     particles grouped by brick (order within a brick arbitrary)
//   k_cell_sort   per brick: cell histogram and starts, then each particle's
//                 rank inside its cell by load index
//   k_permute     the particle fields moved into the sorted order
#include "mpm_device.cuh"

namespace mpm {

template <typename R>
__global__ void k_bin(KGeom<R> g, int nbx, int nby, const R *x0, const R *x1, const R *x2, int n, int *key,
                      int *bcount, unsigned *oob_count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool oob = false;
    int k = -1;
    if (i < n) {
        int cx = cell_of(x0[i], g, 0, oob), cy = cell_of(x1[i], g, 1, oob), cz = cell_of(x2[i], g, 2, oob);
        int b = cx / BRX + nbx * (cy / BRY + nby * (cz / BRZ));
        int lc = (cx % BRX) + BRX * ((cy % BRY) + BRY * (cz % BRZ));
        k = b;
        key[i] = b * BRC + lc;
    }
    unsigned act = __ballot_sync(0xffffffffu, i < n);
    if (i < n) {
        unsigned peers = __match_any_sync(act, k);
        int leader = __ffs(peers) - 1;
        if ((int)(threadIdx.x & 31) == leader) atomicAdd(&bcount[k], __popc(peers));
    }
    unsigned bad = __ballot_sync(0xffffffffu, oob);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(oob_count, __popc(bad));
}

// Exclusive scan of the brick counts in three launches over segments of
// SCAN_SEG bricks: (1) each CTA sums its segment's particles, work items
// (chunks of <= CHUNK particles) and non-empty bricks; (2) one CTA scans the
// segment sums; (3) each CTA scans its segment again in brick order from its
// segment's offsets and writes the brick starts, the work list, the list of
// non-empty bricks, and resets the counters for the next sort.  Every load
// and store of the brick arrays is coalesced.
constexpr int SCAN_T = 1024;                 // threads per CTA
constexpr int SCAN_ITEMS = SCAN_SEG / SCAN_T;  // bricks per thread and segment
static_assert(SCAN_ITEMS * SCAN_T == SCAN_SEG, "scan segment");

struct Tri {
    int c, k, a;   // particles, work items, non-empty bricks
};
__device__ __forceinline__ Tri tri_of(int c) { return Tri{c, (c + CHUNK - 1) / CHUNK, c > 0 ? 1 : 0}; }

// inclusive block-wide scan of (c, k, a) over SCAN_T threads; the block total in *tot
__device__ __forceinline__ Tri block_scan(Tri v, Tri *sh, Tri *tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int c = __shfl_up_sync(0xffffffffu, v.c, o), k = __shfl_up_sync(0xffffffffu, v.k, o),
                  a = __shfl_up_sync(0xffffffffu, v.a, o);
        if (lane >= o) {
            v.c += c;
            v.k += k;
            v.a += a;
        }
    }
    if (lane == 31) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        Tri w = lane < (SCAN_T >> 5) ? sh[lane] : Tri{0, 0, 0};
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int c = __shfl_up_sync(0xffffffffu, w.c, o), k = __shfl_up_sync(0xffffffffu, w.k, o),
                      a = __shfl_up_sync(0xffffffffu, w.a, o);
            if (lane >= o) {
                w.c += c;
                w.k += k;
                w.a += a;
            }
        }
        if (lane < (SCAN_T >> 5)) sh[lane] = w;   // inclusive warp offsets
    }
    __syncthreads();
    if (wid > 0) {
        const Tri b = sh[wid - 1];
        v.c += b.c;
        v.k += b.k;
        v.a += b.a;
    }
    *tot = sh[(SCAN_T >> 5) - 1];
    __syncthreads();   // sh is reused by the next call
    return v;
}

__global__ void __launch_bounds__(SCAN_T) k_scan_up(int nb, const int *__restrict__ bcount, int *part) {
    __shared__ Tri sh[32];
    const int base = blockIdx.x * SCAN_SEG;
    Tri v{0, 0, 0};
#pragma unroll
    for (int r = 0; r < SCAN_ITEMS; r++) {
        const int t = base + r * SCAN_T + threadIdx.x;
        if (t < nb) {
            const Tri q = tri_of(bcount[t]);
            v.c += q.c;
            v.k += q.k;
            v.a += q.a;
        }
    }
    Tri tot;
    block_scan(v, sh, &tot);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = tot.c;
        part[3 * blockIdx.x + 1] = tot.k;
        part[3 * blockIdx.x + 2] = tot.a;
    }
}

// exclusive scan of the nseg segment sums in place; the totals after them
__global__ void __launch_bounds__(SCAN_T) k_scan_mid(int nseg, int *part) {
    __shared__ Tri sh[32];
    Tri carry{0, 0, 0};
    for (int s0 = 0; s0 < nseg; s0 += SCAN_T) {
        const int i = s0 + threadIdx.x;
        const Tri v = i < nseg ? Tri{part[3 * i], part[3 * i + 1], part[3 * i + 2]} : Tri{0, 0, 0};
        Tri tot;
        const Tri inc = block_scan(v, sh, &tot);
        if (i < nseg) {
            part[3 * i] = carry.c + inc.c - v.c;
            part[3 * i + 1] = carry.k + inc.k - v.k;
            part[3 * i + 2] = carry.a + inc.a - v.a;
        }
        carry.c += tot.c;
        carry.k += tot.k;
        carry.a += tot.a;
    }
    if (threadIdx.x == 0) {
        part[3 * nseg] = carry.c;
        part[3 * nseg + 1] = carry.k;
        part[3 * nseg + 2] = carry.a;
    }
}

__global__ void __launch_bounds__(SCAN_T) k_scan_down(int nb, int nseg, int *bcount, int *bstart, int *bcursor,
                                                      WorkItem *work, int *nwork, int cap, int *blist, int *nblist,
                                                      const int *part) {
    __shared__ Tri sh[32];
    const int base = blockIdx.x * SCAN_SEG;
    Tri carry{part[3 * blockIdx.x], part[3 * blockIdx.x + 1], part[3 * blockIdx.x + 2]};
    for (int r = 0; r < SCAN_ITEMS; r++) {
        const int t = base + r * SCAN_T + threadIdx.x;
        const int c = t < nb ? bcount[t] : 0;
        const Tri v = tri_of(c);
        Tri tot;
        const Tri inc = block_scan(v, sh, &tot);
        if (t < nb) {
            const int pbase = carry.c + inc.c - v.c;
            int wbase = carry.k + inc.k - v.k;
            if (c > 0) blist[carry.a + inc.a - v.a] = t;
            bstart[t] = pbase;
            bcursor[t] = 0;
            bcount[t] = 0;
            for (int b = 0; b < c; b += CHUNK) {
                if (wbase < cap) {
                    WorkItem w;
                    w.tile = t;
                    w.begin = pbase + b;
                    w.end = pbase + min(c, b + CHUNK);
                    work[wbase] = w;
                }
                wbase++;
            }
        }
        carry.c += tot.c;
        carry.k += tot.k;
        carry.a += tot.a;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *nwork = min(part[3 * nseg + 1], cap);
        *nblist = part[3 * nseg + 2];
        bstart[nb] = part[3 * nseg];
    }
}

__global__ void k_scatter(const int *key, int n, const int *bstart, int *bcursor, int *tmp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned act = __ballot_sync(0xffffffffu, i < n);
    if (i >= n) return;
    int k = key[i] / BRC;
    unsigned peers = __match_any_sync(act, k);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int rank = __popc(peers & ((1u << lane) - 1));
    int base = 0;
    if (lane == leader) base = atomicAdd(&bcursor[k], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    tmp[bstart[k] + base + rank] = i;
}

// One CTA per brick.  tmp holds the brick's particles in arbitrary order;
// writes perm (sorted by cell, then load index) and the brick's cell starts.
// tmp2 is scratch where each cell's particles become contiguous.
__global__ void __launch_bounds__(BRC) k_cell_sort(const int *bstart, const int *key, const int *pid,
                                                   const int *tmp, int *tmp2, int *perm, int *cstart) {
    __shared__ int s_cnt[BRC];
    __shared__ int s_cur[BRC];
    __shared__ int s_start[BRC + 1];
    const int b = blockIdx.x;
    const int lo = bstart[b], hi = bstart[b + 1];
    const int lc = threadIdx.x;
    int *cs = cstart + (size_t)b * (BRC + 1);
    if (lo == hi) {   // an empty brick (uniform across the CTA): every cell starts at lo
        cs[lc] = lo;
        if (lc == 0) cs[BRC] = hi;
        return;
    }
    s_cnt[lc] = 0;
    s_cur[lc] = 0;
    __syncthreads();
    for (int j = lo + lc; j < hi; j += BRC) atomicAdd(&s_cnt[key[tmp[j]] % BRC], 1);
    __syncthreads();
    {   // exclusive scan of the BRC cell counts: warp scans, then the warp offsets
        static_assert(BRC % 32 == 0 && BRC / 32 <= 32, "cell scan layout");
        const int lane = lc & 31, wid = lc >> 5;
        int v = s_cnt[lc];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        __shared__ int s_w[BRC / 32];
        if (lane == 31) s_w[wid] = v;
        __syncthreads();
        int off = 0;
        for (int w = 0; w < wid; w++) off += s_w[w];
        s_start[lc + 1] = off + v;
        if (lc == 0) s_start[0] = 0;
    }
    __syncthreads();
    cs[lc] = lo + s_start[lc];
    if (lc == 0) cs[BRC] = hi;
    for (int j = lo + lc; j < hi; j += BRC) {
        const int i = tmp[j];
        const int c = key[i] % BRC;
        tmp2[lo + s_start[c] + atomicAdd(&s_cur[c], 1)] = i;
    }
    __syncthreads();
    // rank inside the cell: the number of the cell's particles with a smaller load index
    for (int j = lo + lc; j < hi; j += BRC) {
        const int i = tmp2[j];
        const int c = key[i] % BRC;
        const int me = pid[i];
        const int c0 = lo + s_start[c], c1 = lo + s_start[c + 1];
        int r = 0;
        for (int q = c0; q < c1; q++) r += (pid[tmp2[q]] < me);
        perm[c0 + r] = i;
    }
}

// dst[j] = src[perm[j]] for all real fields and the two int fields.  The
// two buffers never overlap; eight fields are loaded before they are stored
// so that a thread keeps eight gathers in flight.
template <typename R>
__global__ void k_permute(const R *__restrict__ src, R *__restrict__ dst, const int *__restrict__ perm, int n,
                          int nreal, size_t N, int skip_lo, int skip_hi) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const size_t i = (size_t)perm[j];
    // fields [skip_lo, skip_hi) are not moved (no kernel of the context reads them)
    const int nmove = nreal - (skip_hi - skip_lo);
    auto field = [&](int k) { return k < skip_lo ? k : k + (skip_hi - skip_lo); };
    int q = 0;
    for (; q + 8 <= nmove; q += 8) {
        R v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = __ldg(src + (size_t)field(q + k) * N + i);
#pragma unroll
        for (int k = 0; k < 8; k++) dst[(size_t)field(q + k) * N + j] = v[k];
    }
    for (; q < nmove; q++) dst[(size_t)field(q) * N + j] = __ldg(src + (size_t)field(q) * N + i);
    const int *si = (const int *)(src + (size_t)nreal * N);
    int *di = (int *)(dst + (size_t)nreal * N);
    const int a0 = __ldg(si + i), a1 = __ldg(si + N + i);
    di[j] = a0;
    di[N + j] = a1;
}

template <typename R>
static mpm_status sort_impl(mpm_ctx *c) {
    int n = (int)c->num;
    if (n == 0) return MPM_OK;
    KGeom<R> g;
    for (int d = 0; d < 3; d++) {
        g.xmin[d] = (R)c->g.xmin[d];
        g.dx[d] = (R)c->g.dx[d];
        g.inv_dx[d] = (R)(1.0 / c->g.dx[d]);
        g.nel[d] = c->g.nel[d];
        g.nnc[d] = c->g.nnc[d];
        g.ntile[d] = c->g.ntile[d];
    }
    g.nodec = c->g.nodec;
    const R *src = (const R *)c->pbuf[c->cur];
    R *dst = (R *)c->pbuf[c->cur ^ 1];
    size_t N = c->pstride;
    const int *pid = (const int *)(src + c->nreal * N) + N;
    int nb = (n + 255) / 256;
    timer_begin(c, K_BIN);
    k_bin<R><<<nb, 256, 0, c->stream>>>(g, c->g.nbrick[0], c->g.nbrick[1], src, src + N, src + 2 * N, n, c->d_key,
                                        c->d_tcount, &c->d_ctl->err_oob);
    timer_end(c, K_BIN);
    timer_begin(c, K_SCAN);
    {
        const int nseg = (c->g.nbricks + SCAN_SEG - 1) / SCAN_SEG;
        k_scan_up<<<nseg, SCAN_T, 0, c->stream>>>(c->g.nbricks, c->d_tcount, c->d_scanpart);
        k_scan_mid<<<1, SCAN_T, 0, c->stream>>>(nseg, c->d_scanpart);
        k_scan_down<<<nseg, SCAN_T, 0, c->stream>>>(c->g.nbricks, nseg, c->d_tcount, c->d_tstart, c->d_tcursor,
                                                    c->d_work, c->d_nwork, c->nwork_cap, c->d_blist, c->d_nblist,
                                                    c->d_scanpart);
        c->launches += 3;
    }
    timer_end(c, K_SCAN);
    timer_begin(c, K_SCATTER);
    k_scatter<<<nb, 256, 0, c->stream>>>(c->d_key, n, c->d_tstart, c->d_tcursor, c->d_tmp);
    k_cell_sort<<<c->g.nbricks, BRC, 0, c->stream>>>(c->d_tstart, c->d_key, pid, c->d_tmp, c->d_perm2, c->d_perm,
                                                      c->d_cstart);
    timer_end(c, K_SCATTER);
    timer_begin(c, K_PERMUTE);
    // a Tait-fluid context keeps J - 1 in the first F field and never reads the other eight
    const int skip_lo = c->fluid_j ? 7 : 0, skip_hi = c->fluid_j ? 15 : 0;
    k_permute<R><<<nb, 256, 0, c->stream>>>(src, dst, c->d_perm, n, c->nreal, N, skip_lo, skip_hi);
    timer_end(c, K_PERMUTE);
    c->launches += 5;
    c->cur ^= 1;
    c->resorts++;
    c->steps_since_sort = 0;
    return check_launch(c);
}

mpm_status sort_particles(mpm_ctx *c) { return c->precision == 64 ? sort_impl<double>(c) : sort_impl<float>(c); }

}  // namespace mpm
