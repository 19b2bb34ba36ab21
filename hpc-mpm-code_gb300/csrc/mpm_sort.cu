// Particle binning and the tile counting sort.
//
// MeshPointLinklist (module/material_point.cpp:52-78) builds a per-cell
// linked list every step.  Here every kernel recomputes a particle's cell
// from its position (that is the per-step binning), and the particles are
// physically regrouped by 8x8x8 tile with a counting sort every
// resort_period steps so that a CTA's particles share one staging box.
// The P2G sums are fixed point, so the order of particles inside and across
// tiles does not change any result.
#include "mpm_device.cuh"

namespace mpm {

template <typename R>
__global__ void k_bin(KGeom<R> g, const R *x0, const R *x1, const R *x2, int n, int *key, int *tcount,
                      unsigned *oob_count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool oob = false;
    int k = -1;
    if (i < n) {
        int cx = cell_of(x0[i], g, 0, oob), cy = cell_of(x1[i], g, 1, oob), cz = cell_of(x2[i], g, 2, oob);
        k = cx / TILE + g.ntile[0] * (cy / TILE + g.ntile[1] * (cz / TILE));
        key[i] = k;
    }
    // warp-aggregated histogram
    unsigned act = __ballot_sync(0xffffffffu, i < n);
    if (i < n) {
        unsigned peers = __match_any_sync(act, k);
        int leader = __ffs(peers) - 1;
        if ((int)(threadIdx.x & 31) == leader) atomicAdd(&tcount[k], __popc(peers));
    }
    unsigned bad = __ballot_sync(0xffffffffu, oob);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(oob_count, __popc(bad));
}

// One CTA: exclusive scan of the tile counts, the work list of <= CHUNK
// particle chunks per tile, and the reset of the counters for the next sort.
__global__ void __launch_bounds__(1024) k_scan(int ntiles, int *tcount, int *tstart, int *tcursor, WorkItem *work,
                                               int *nwork, int cap) {
    __shared__ int s_cnt[1024];
    __shared__ int s_chk[1024];
    const int T = blockDim.x;
    const int per = (ntiles + T - 1) / T;
    const int lo = threadIdx.x * per, hi = min(lo + per, ntiles);
    int csum = 0, ksum = 0;
    for (int t = lo; t < hi; t++) {
        int c = tcount[t];
        csum += c;
        ksum += (c + CHUNK - 1) / CHUNK;
    }
    s_cnt[threadIdx.x] = csum;
    s_chk[threadIdx.x] = ksum;
    __syncthreads();
    // Hillis-Steele inclusive scan over the per-thread sums
    for (int off = 1; off < T; off <<= 1) {
        int a = threadIdx.x >= off ? s_cnt[threadIdx.x - off] : 0;
        int b = threadIdx.x >= off ? s_chk[threadIdx.x - off] : 0;
        __syncthreads();
        s_cnt[threadIdx.x] += a;
        s_chk[threadIdx.x] += b;
        __syncthreads();
    }
    int pbase = s_cnt[threadIdx.x] - csum;
    int wbase = s_chk[threadIdx.x] - ksum;
    for (int t = lo; t < hi; t++) {
        int c = tcount[t];
        tstart[t] = pbase;
        tcursor[t] = 0;
        tcount[t] = 0;
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
    if (threadIdx.x == T - 1) *nwork = min(s_chk[T - 1], cap);
}

__global__ void k_scatter(const int *key, int n, const int *tstart, int *tcursor, int *perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned act = __ballot_sync(0xffffffffu, i < n);
    if (i >= n) return;
    int k = key[i];
    unsigned peers = __match_any_sync(act, k);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int rank = __popc(peers & ((1u << lane) - 1));
    int base = 0;
    if (lane == leader) base = atomicAdd(&tcursor[k], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    perm[tstart[k] + base + rank] = i;
}

// dst[j] = src[perm[j]] for all 24 real fields and the two int fields.
template <typename R>
__global__ void k_permute(const R *src, R *dst, const int *perm, int n) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int i = perm[j];
    size_t N = (size_t)n;
#pragma unroll 4
    for (int f = 0; f < 24; f++) dst[f * N + j] = src[f * N + i];
    const int *si = (const int *)(src + 24 * N);
    int *di = (int *)(dst + 24 * N);
    di[j] = si[i];
    di[N + j] = si[N + i];
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
    size_t N = (size_t)n;
    int nb = (n + 255) / 256;
    timer_begin(c, K_BIN);
    k_bin<R><<<nb, 256, 0, c->stream>>>(g, src, src + N, src + 2 * N, n, c->d_key, c->d_tcount, &c->d_ctl->err_oob);
    timer_end(c, K_BIN);
    timer_begin(c, K_SCAN);
    k_scan<<<1, 1024, 0, c->stream>>>(c->g.ntiles, c->d_tcount, c->d_tstart, c->d_tcursor, c->d_work, c->d_nwork,
                                      c->nwork_cap);
    timer_end(c, K_SCAN);
    timer_begin(c, K_SCATTER);
    k_scatter<<<nb, 256, 0, c->stream>>>(c->d_key, n, c->d_tstart, c->d_tcursor, c->d_perm);
    timer_end(c, K_SCATTER);
    timer_begin(c, K_PERMUTE);
    k_permute<R><<<nb, 256, 0, c->stream>>>(src, dst, c->d_perm, n);
    timer_end(c, K_PERMUTE);
    c->launches += 4;
    c->cur ^= 1;
    c->resorts++;
    c->steps_since_sort = 0;
    return check_launch(c);
}

mpm_status sort_particles(mpm_ctx *c) { return c->precision == 64 ? sort_impl<double>(c) : sort_impl<float>(c); }

}  // namespace mpm
