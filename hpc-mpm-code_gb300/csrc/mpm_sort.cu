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
//   k_scan        brick starts, work-item list (chunks of <= CHUNK particles)
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

// One CTA: exclusive scan of the brick counts, the work list of <= CHUNK
// particle chunks per brick, and the reset of the counters for the next sort.
__global__ void __launch_bounds__(1024) k_scan(int nb, int *bcount, int *bstart, int *bcursor, WorkItem *work,
                                               int *nwork, int cap, int *blist, int *nblist) {
    __shared__ int s_cnt[1024];
    __shared__ int s_chk[1024];
    __shared__ int s_act[1024];
    const int T = blockDim.x;
    const int per = (nb + T - 1) / T;
    const int lo = threadIdx.x * per, hi = min(lo + per, nb);
    int csum = 0, ksum = 0, asum = 0;
    for (int t = lo; t < hi; t++) {
        int c = bcount[t];
        csum += c;
        ksum += (c + CHUNK - 1) / CHUNK;
        asum += c > 0;
    }
    s_cnt[threadIdx.x] = csum;
    s_chk[threadIdx.x] = ksum;
    s_act[threadIdx.x] = asum;
    __syncthreads();
    for (int off = 1; off < T; off <<= 1) {
        int a = threadIdx.x >= off ? s_cnt[threadIdx.x - off] : 0;
        int b = threadIdx.x >= off ? s_chk[threadIdx.x - off] : 0;
        int d = threadIdx.x >= off ? s_act[threadIdx.x - off] : 0;
        __syncthreads();
        s_cnt[threadIdx.x] += a;
        s_chk[threadIdx.x] += b;
        s_act[threadIdx.x] += d;
        __syncthreads();
    }
    int pbase = s_cnt[threadIdx.x] - csum;
    int wbase = s_chk[threadIdx.x] - ksum;
    int abase = s_act[threadIdx.x] - asum;
    for (int t = lo; t < hi; t++) {
        int c = bcount[t];
        if (c > 0) blist[abase++] = t;
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
        pbase += c;
    }
    if (threadIdx.x == T - 1) {
        *nwork = min(s_chk[T - 1], cap);
        *nblist = s_act[T - 1];
        bstart[nb] = s_cnt[T - 1];
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
    s_cnt[lc] = 0;
    s_cur[lc] = 0;
    __syncthreads();
    for (int j = lo + lc; j < hi; j += BRC) atomicAdd(&s_cnt[key[tmp[j]] % BRC], 1);
    __syncthreads();
    if (lc == 0) {
        int acc = 0;
        for (int c = 0; c < BRC; c++) {
            s_start[c] = acc;
            acc += s_cnt[c];
        }
        s_start[BRC] = acc;
    }
    __syncthreads();
    int *cs = cstart + (size_t)b * (BRC + 1);
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
    k_scan<<<1, 1024, 0, c->stream>>>(c->g.nbricks, c->d_tcount, c->d_tstart, c->d_tcursor, c->d_work, c->d_nwork,
                                      c->nwork_cap, c->d_blist, c->d_nblist);
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
