// Learned preconditioner network: forward, backward (data and weight
// gradients) and Adam training, with the 3x3x3 convolutions on tcgen05
// tensor cores (BF16 operands, FP32 accumulators in tensor memory).
//
// No counterpart in the reference: HPC-MPM-Code solves its linear systems
// with GPBiCGSafe or PETSc (module/solver/solver.cpp:19-141,
// module/solver/crsmat.cpp:338-686).  The network is the right
// preconditioner of the flexible conjugate gradient solver in
// mpm_implicit.cu.
//
// Convolution as implicit GEMM: a CTA owns 128 output nodes (one TMEM lane
// each); for every one of the 27 taps its 128 threads gather the tap's input
// rows (channels-last, 16-byte vectors) into a K-major shared-memory tile
// while the tensor core multiplies the previous tap's tile by that tap's
// weights (all 27 weight tiles stay in shared memory).  Two tile buffers, an
// mbarrier per buffer completed by tcgen05.commit.  The weight gradient
// dW[t][ci][co] = sum_v x[gather(v, t)][ci] g[v][co] runs as a GEMM with the
// (tap, ci) pairs as M (128 per MMA), the output channels as N and the nodes
// as K: the gathered input is written transposed into shared memory.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include <cuda.h>

#include "mpm_nn.cuh"
#include "mpm_tc.cuh"

typedef __nv_bfloat16 bf16;

using namespace mpm;
using namespace mpm::nn;

#define CKN(call)                                                                                                      \
    do {                                                                                                               \
        cudaError_t _e = (call);                                                                                       \
        if (_e != cudaSuccess) {                                                                                       \
            fprintf(stderr, "mpm_gb300 (nn): %s failed: %s\n", #call, cudaGetErrorString(_e));                         \
            return _e == cudaErrorMemoryAllocation ? MPM_ERR_OOM : MPM_ERR_CUDA;                                       \
        }                                                                                                              \
    } while (0)

namespace mpm {
namespace nn {

int64_t w_offset(int l) {
    int64_t o = 0;
    for (int i = 0; i < l; i++) o += 27LL * CIN[i] * COUT[i] + COUT[i];
    return o;
}
int64_t b_offset(int l) { return w_offset(l) + 27LL * CIN[l] * COUT[l]; }
int64_t w5_offset() { return w_offset(NCONV); }
int64_t b5_offset() { return w5_offset() + 48; }
int64_t param_count() { return b5_offset() + 3; }

enum Mode { S1 = 0, S2 = 1, S1T = 2, S2T = 3 };
constexpr unsigned TC_WAIT = 1u << 22;   // try_wait polls before a wait gives up

struct Lvl {
    int n[3];
    int64_t v;
};

// Source row of output node (b, o) for tap t, or -1 (zero padding).
template <int MODE>
__device__ __forceinline__ int64_t gather_src(int b, int ox, int oy, int oz, int t, const Lvl &in) {
    const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
    int ix, iy, iz;
    if (MODE == S1) {
        ix = ox + dx;
        iy = oy + dy;
        iz = oz + dz;
    } else if (MODE == S2) {
        ix = 2 * ox + dx;
        iy = 2 * oy + dy;
        iz = 2 * oz + dz;
    } else if (MODE == S1T) {
        ix = ox - dx;
        iy = oy - dy;
        iz = oz - dz;
    } else {
        const int tx = ox - dx, ty = oy - dy, tz = oz - dz;
        if ((tx | ty | tz) & 1) return -1;
        ix = tx >> 1;
        iy = ty >> 1;
        iz = tz >> 1;
    }
    if (ix < 0 || iy < 0 || iz < 0 || ix >= in.n[0] || iy >= in.n[1] || iz >= in.n[2]) return -1;
    return (int64_t)b * in.v + ix + (int64_t)in.n[0] * (iy + (int64_t)in.n[1] * iz);
}

// (sample, x, y, z) of a row; rows are below 2^31 (checked when the network
// is created), so 32-bit divisions do
__device__ __forceinline__ void row_coords(int64_t row, const Lvl &L, int &b, int &x, int &y, int &z) {
    const int r = (int)row, lv = (int)L.v;
    b = r / lv;
    const int v = r - b * lv;
    const int q = v / L.n[0];
    x = v - q * L.n[0];
    z = q / L.n[1];
    y = q - z * L.n[1];
}

__device__ __forceinline__ void unpack8(const uint4 &u, float *f) {
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float2 t = __bfloat1622float2(h[i]);
        f[2 * i] = t.x;
        f[2 * i + 1] = t.y;
    }
}

__device__ __forceinline__ uint4 pack8(const float *f) {
    uint4 u;
    __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    return u;
}

// ------------------------------------------------------------------ conv
struct ConvArgs {
    const bf16 *in;     // [rows_in][K]
    bf16 *out;          // [rows][N]
    const bf16 *w;      // 27 canonical N x K tiles
    const float *bias;  // [N] or null
    const bf16 *add;    // [rows][N] or null: added before the activation
    const bf16 *mask;   // [rows][N] or null: output zeroed where mask <= 0
    int relu;
    Lvl lin, lout;
    int64_t rows;       // batch * lout.v
    int *err;
};

// Taps gathered per pipeline stage: a whole 3x3 plane (9) when the stage
// fits, else a row of 3.
template <int K, int N>
__host__ __device__ constexpr int conv_tg() {
    return (27u * N * K * 2 + 2u * 9 * 128 * K * 2 <= 200u * 1024) ? 9 : 3;
}

template <int K, int N>
__host__ __device__ constexpr size_t conv_smem() {
    return 27u * N * K * 2 + 2u * conv_tg<K, N>() * 128 * K * 2;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit_wait() {
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// Per tile of 128 output nodes the 27 taps are processed in groups of TG:
// every thread gathers its row of the group's TG input tiles with 16-byte
// cp.async copies (zero-filled for padding, no registers held), so TG taps'
// loads are in flight at once; then one thread issues the group's MMAs and
// commits them to the stage's mbarrier.  Two stages: a stage is refilled
// only after the MMAs that read it completed.
template <int K, int N, int MODE>
__global__ void __launch_bounds__(128) k_conv_tc(ConvArgs a) {
    constexpr int TG = conv_tg<K, N>();
    constexpr int NG = 27 / TG;
    constexpr uint32_t WT = (uint32_t)N * K * 2;        // one tap's weight tile
    constexpr uint32_t WB = 27u * WT;
    constexpr uint32_t AB = 128u * K * 2;               // one tap's A tile
    constexpr uint32_t SB = TG * AB;                    // one stage
    constexpr uint32_t TCOLS = N < 32 ? 32 : N;
    constexpr uint32_t IDESC = tc::idesc_bf16(128, N);
    constexpr uint32_t SBO = K * 16;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ unsigned long long bar[2], wbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tc::tmem_alloc(&tslot, TCOLS);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&wbar, 1);
        fence_mbar_init();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    // the 27 weight tiles by bulk copies, waited for before the first MMA
    if (tid == 0) {
        mbar_expect_tx(&wbar, WB);
        constexpr uint32_t WCH = 32768;
        for (uint32_t o = 0; o < WB; o += WCH)
            bulk_g2s(smem + o, reinterpret_cast<const unsigned char *>(a.w) + o, WB - o < WCH ? WB - o : WCH, &wbar);
    }
    bool wready = false;
    const uint32_t taddr = tslot;
    const uint32_t sw = smem_addr(smem), sa = sw + WB;
    // this thread's row inside a tap tile: (row / 8) * SBO + (row % 8) * 16
    const uint32_t rowoff = (uint32_t)(tid >> 3) * SBO + (uint32_t)(tid & 7) * 16;
    const int64_t ntile = (a.rows + 127) / 128;
    uint32_t it = 0;   // stage uses so far
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int64_t row = tile * 128 + tid;
        const bool valid = row < a.rows;
        int b = 0, ox = 0, oy = 0, oz = 0;
        if (valid) row_coords(row, a.lout, b, ox, oy, oz);
        for (int g = 0; g < NG; g++) {
            const uint32_t s = it & 1;
            bool mine = true;
            if (it >= 2) mine = mbar_wait_bounded(&bar[s], ((it >> 1) - 1) & 1, TC_WAIT);
            if (!__syncthreads_and(mine)) {
                ok = false;
                break;
            }
#pragma unroll
            for (int tl = 0; tl < TG; tl++) {
                const int t = g * TG + tl;
                const int64_t src = valid ? gather_src<MODE>(b, ox, oy, oz, t, a.lin) : -1;
                const bf16 *in = a.in + (src >= 0 ? src : 0) * K;
                const uint32_t dst = sa + s * SB + tl * AB + rowoff;
#pragma unroll
                for (int kc = 0; kc < K / 8; kc++) cp_async16(dst + kc * 128, in + kc * 8, src >= 0);
            }
            cp_async_commit_wait();
            tc::fence_async_smem();
            tc::fence_before();
            if (!wready) {
                wready = true;
                if (!__syncthreads_and(mbar_wait_bounded(&wbar, 0, TC_WAIT))) {
                    ok = false;
                    break;
                }
            }
            __syncthreads();
            if (tid == 0) {
                tc::fence_after();
#pragma unroll
                for (int tl = 0; tl < TG; tl++) {
                    const int t = g * TG + tl;
#pragma unroll
                    for (int kk = 0; kk < K / 16; kk++) {
                        const uint64_t ad = tc::sdesc(sa + s * SB + tl * AB + kk * 256, 128, SBO);
                        const uint64_t bd = tc::sdesc(sw + t * WT + kk * 256, 128, SBO);
                        tc::mma_bf16(taddr, ad, bd, IDESC, (t | kk) != 0);
                    }
                }
                tc::mma_commit(&bar[s]);
            }
            it++;
        }
        if (!ok) break;
        const bool done = mbar_wait_bounded(&bar[(it - 1) & 1], ((it - 1) >> 1) & 1, TC_WAIT);
        if (!__syncthreads_and(done)) {
            ok = false;
            break;
        }
        tc::fence_after();
        float acc[N];
#pragma unroll
        for (int c = 0; c < N / 16; c++) tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + c * 16, acc + c * 16);
        if (valid) {
            if (a.bias) {
#pragma unroll
                for (int c = 0; c < N; c++) acc[c] += __ldg(a.bias + c);
            }
            if (a.add) {
                const uint4 *ap = reinterpret_cast<const uint4 *>(a.add + row * N);
#pragma unroll
                for (int c = 0; c < N / 8; c++) {
                    float f[8];
                    unpack8(__ldg(ap + c), f);
#pragma unroll
                    for (int i = 0; i < 8; i++) acc[c * 8 + i] += f[i];
                }
            }
            if (a.relu) {
#pragma unroll
                for (int c = 0; c < N; c++) acc[c] = fmaxf(acc[c], 0.0f);
            }
            if (a.mask) {
                const uint4 *mp = reinterpret_cast<const uint4 *>(a.mask + row * N);
#pragma unroll
                for (int c = 0; c < N / 8; c++) {
                    float f[8];
                    unpack8(__ldg(mp + c), f);
#pragma unroll
                    for (int i = 0; i < 8; i++)
                        if (!(f[i] > 0.0f)) acc[c * 8 + i] = 0.0f;
                }
            }
            uint4 *op = reinterpret_cast<uint4 *>(a.out + row * N);
#pragma unroll
            for (int c = 0; c < N / 8; c++) op[c] = pack8(acc + c * 8);
        }
        tc::fence_before();
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) atomicAdd(a.err, 1);
        if (it > 0) mbar_wait_bounded(&bar[(it - 1) & 1], ((it - 1) >> 1) & 1, TC_WAIT);
        mbar_wait_bounded(&wbar, 0, TC_WAIT);
    }
    if (!wready) mbar_wait_bounded(&wbar, 0, TC_WAIT);   // a block without tiles still lets its copy land
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::tmem_dealloc(taddr, TCOLS);
}

// ------------------------------------------------- halo-tiled convolution
// Forward convolutions (S1, S2) as an implicit GEMM over a shared-memory halo
// tile loaded by TMA.  An output tile is 8 (x) x 16 (y) x 1 (z) nodes = the
// 128 rows of one MMA, row m = x + 8 y.  Its input halo (S1: 10 x 18 x 3
// nodes; S2: 17 x 33 x 3) is brought in by one tensor copy per 8-channel
// chunk (a 5-D tensor map per chunk: 8 channels, x, y, z, sample; zero fill
// outside the grid), which lands as [z][y][x] 16-byte entries.  For every tap
// the A operand is then the same canonical K-major no-swizzle matrix at a
// shifted start address: 8 consecutive x entries form a core matrix, the
// chunk stride is the leading byte offset and the y stride (2 y strides for
// S2) the stride byte offset.  For S2 the even and odd x positions are two
// copies with a traversal stride of 2, so that the stride-2 rows of a tap are
// again consecutive entries.  Each input node is read about 4 times per tile
// instead of 27 times, one thread issues all copies, and with two halo
// buffers the copy of the next tile overlaps the MMAs and the epilogue of the
// current one.
template <int MODE>
struct Halo {
    static constexpr int TX = 8, TY = 16;
    static constexpr int XE = MODE == S1 ? 10 : 9;     // x entries per row and copy
    static constexpr int HY = MODE == S1 ? 18 : 33;
    static constexpr int HZ = 3;
    static constexpr uint32_t COPY = 16u * XE * HY * HZ;            // bytes of one tensor copy
    static constexpr uint32_t BLK = (COPY + 127u) / 128u * 128u;   // its 128-byte aligned slot
    static constexpr uint32_t CHUNK = (MODE == S1 ? 1u : 2u) * BLK; // one 8-channel chunk (S2: even, odd)
    static constexpr uint32_t RS = 16u * XE;                        // y stride
    static constexpr uint32_t PS = RS * HY;                         // z stride
};

template <int K, int MODE>
__host__ __device__ constexpr uint32_t halo_bytes() {
    return (uint32_t)(K / 8) * Halo<MODE>::CHUNK;
}

template <int K, int N, int MODE>
__host__ __device__ constexpr int halo_nbuf() {
    return 27u * N * K * 2 + 2u * halo_bytes<K, MODE>() <= 200u * 1024 ? 2 : 1;
}

template <int K, int N, int MODE>
__host__ __device__ constexpr size_t halo_smem() {
    return 27u * N * K * 2 + (size_t)halo_nbuf<K, N, MODE>() * halo_bytes<K, MODE>() + 128;
}

struct HaloMaps {
    CUtensorMap m[8];   // one per 8-channel chunk of the input
};

__device__ __forceinline__ void tma_load5(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3, int c4,
                                          unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_addr(bar))
        : "memory");
}

template <int K, int N, int MODE>
__global__ void __launch_bounds__(128) k_conv_halo(ConvArgs a, const __grid_constant__ HaloMaps maps) {
    using H = Halo<MODE>;
    constexpr int KC = K / 8;
    constexpr int NBUF = halo_nbuf<K, N, MODE>();
    constexpr uint32_t WT = (uint32_t)N * K * 2;
    constexpr uint32_t WB = 27u * WT;
    constexpr uint32_t HB = halo_bytes<K, MODE>();
    constexpr uint32_t LBO = H::CHUNK;
    constexpr uint32_t SBO_A = MODE == S1 ? H::RS : 2 * H::RS;
    constexpr uint32_t SBO_W = K * 16;
    constexpr uint32_t TX_BYTES = (uint32_t)KC * (MODE == S1 ? 1u : 2u) * H::COPY;
    constexpr uint32_t TCOLS = N < 32 ? 32 : N;
    constexpr uint32_t IDESC = tc::idesc_bf16(128, N);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ unsigned long long bar, full[2], wbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5;
    // halo buffers first, 128-byte aligned (tensor copy destinations), then the weights
    const uint32_t sbase = (smem_addr(smem_raw) + 127u) & ~127u;
    unsigned char *smem = smem_raw + (sbase - smem_addr(smem_raw));
    const uint32_t sh = sbase, sw = sbase + NBUF * HB;
    if (warp == 0) tc::tmem_alloc(&tslot, TCOLS);
    if (tid == 0) {
        mbar_init(&bar, 1);
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&wbar, 1);
        fence_mbar_init();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    // the 27 weight tiles by bulk copies (one thread, in flight with the
    // first halo copy; waited for before the first MMA)
    if (tid == 0) {
        mbar_expect_tx(&wbar, WB);
        constexpr uint32_t WCH = 32768;
        for (uint32_t o = 0; o < WB; o += WCH)
            bulk_g2s(smem + NBUF * HB + o, reinterpret_cast<const unsigned char *>(a.w) + o, WB - o < WCH ? WB - o : WCH,
                     &wbar);
    }
    const uint32_t taddr = tslot;
    const int ntx = (a.lout.n[0] + H::TX - 1) / H::TX, nty = (a.lout.n[1] + H::TY - 1) / H::TY;
    const int64_t per_b = (int64_t)ntx * nty * a.lout.n[2];
    const int64_t ntile = (a.rows / a.lout.v) * per_b;
    auto coords = [&](int64_t tile, int &b, int &x0, int &y0, int &z0) {
        b = (int)(tile / per_b);
        int64_t r = tile - (int64_t)b * per_b;
        x0 = (int)(r % ntx) * H::TX;
        r /= ntx;
        y0 = (int)(r % nty) * H::TY;
        z0 = (int)(r / nty);
    };
    // thread 0 only: the halo of `tile` into buffer `buf`
    auto issue = [&](int64_t tile, int buf) {
        int b, x0, y0, z0;
        coords(tile, b, x0, y0, z0);
        const uint32_t dst = sh + (uint32_t)buf * HB;
        mbar_expect_tx(&full[buf], TX_BYTES);
#pragma unroll
        for (int kc = 0; kc < KC; kc++) {
            if (MODE == S1) {
                tma_load5(dst + kc * LBO, &maps.m[kc], 0, x0 - 1, y0 - 1, z0 - 1, b, &full[buf]);
            } else {
                tma_load5(dst + kc * LBO, &maps.m[kc], 0, 2 * x0 - 1, 2 * y0 - 1, 2 * z0 - 1, b, &full[buf]);
                tma_load5(dst + kc * LBO + H::BLK, &maps.m[kc], 0, 2 * x0, 2 * y0 - 1, 2 * z0 - 1, b, &full[buf]);
            }
        }
    };
    uint32_t iss0 = 0u, iss1 = 0u, con0 = 0u, con1 = 0u;   // copies issued into / consumed from each buffer
    uint32_t i = 0;
    bool ok = true, mma_pending = false;
    int64_t tile = blockIdx.x;
    if (tile < ntile) {
        if (tid == 0) issue(tile, 0);
        iss0++;
    }
    ok = __syncthreads_and(mbar_wait_bounded(&wbar, 0, TC_WAIT));
    if (!ok) tile = ntile;
    for (; tile < ntile; tile += gridDim.x, i++) {
        const int buf = NBUF == 2 ? (int)(i & 1) : 0;
        const int64_t next = tile + gridDim.x;
        // the other buffer was last read by the MMAs of the previous tile,
        // which completed before that tile's epilogue
        if (NBUF == 2 && next < ntile) {
            if (tid == 0) issue(next, buf ^ 1);
            if (buf) iss0++;
            else iss1++;
        }
        const bool landed = mbar_wait_bounded(&full[buf], (buf ? con1 : con0) & 1u, TC_WAIT);
        if (buf) con1++;
        else con0++;
        if (!__syncthreads_and(landed)) {
            ok = false;
            break;
        }
        if (tid == 0) {
            tc::fence_after();
            const uint32_t cur = sh + (uint32_t)buf * HB;
#pragma unroll
            for (int t = 0; t < 27; t++) {
                const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
                uint32_t base = cur + (uint32_t)(dz + 1) * H::PS + (uint32_t)(dy + 1) * H::RS;
                if (MODE == S1) base += (uint32_t)(dx + 1) * 16u;
                else base += dx == 0 ? H::BLK : (dx > 0 ? 16u : 0u);
#pragma unroll
                for (int kk = 0; kk < K / 16; kk++) {
                    const uint64_t ad = tc::sdesc(base + kk * 2 * LBO, LBO, SBO_A);
                    const uint64_t bd = tc::sdesc(sw + t * WT + kk * 256, 128, SBO_W);
                    tc::mma_bf16(taddr, ad, bd, IDESC, (t | kk) != 0);
                }
            }
            tc::mma_commit(&bar);
        }
        mma_pending = true;
        const bool done = mbar_wait_bounded(&bar, i & 1, TC_WAIT);
        if (!__syncthreads_and(done)) {
            ok = false;
            break;
        }
        mma_pending = false;
        if (NBUF == 1 && next < ntile) {   // the MMAs are done with the only buffer
            if (tid == 0) issue(next, 0);
            iss0++;
        }
        tc::fence_after();
        float acc[N];
#pragma unroll
        for (int c = 0; c < N / 16; c++) tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + c * 16, acc + c * 16);
        int b, x0, y0, z0;
        coords(tile, b, x0, y0, z0);
        const int ox = x0 + (tid & 7), oy = y0 + (tid >> 3);
        if (ox < a.lout.n[0] && oy < a.lout.n[1]) {
            const int64_t row = (int64_t)b * a.lout.v + ox + (int64_t)a.lout.n[0] * (oy + (int64_t)a.lout.n[1] * z0);
            if (a.bias) {
#pragma unroll
                for (int c = 0; c < N; c++) acc[c] += __ldg(a.bias + c);
            }
            if (a.add) {
                const uint4 *ap = reinterpret_cast<const uint4 *>(a.add + row * N);
#pragma unroll
                for (int c = 0; c < N / 8; c++) {
                    float f[8];
                    unpack8(__ldg(ap + c), f);
#pragma unroll
                    for (int e = 0; e < 8; e++) acc[c * 8 + e] += f[e];
                }
            }
            if (a.relu) {
#pragma unroll
                for (int c = 0; c < N; c++) acc[c] = fmaxf(acc[c], 0.0f);
            }
            if (a.mask) {
                const uint4 *mp = reinterpret_cast<const uint4 *>(a.mask + row * N);
#pragma unroll
                for (int c = 0; c < N / 8; c++) {
                    float f[8];
                    unpack8(__ldg(mp + c), f);
#pragma unroll
                    for (int e = 0; e < 8; e++)
                        if (!(f[e] > 0.0f)) acc[c * 8 + e] = 0.0f;
                }
            }
            uint4 *op = reinterpret_cast<uint4 *>(a.out + row * N);
#pragma unroll
            for (int c = 0; c < N / 8; c++) op[c] = pack8(acc + c * 8);
        }
        tc::fence_before();
        __syncthreads();
    }
    if (!ok) {
        if (tid == 0) {
            atomicAdd(a.err, 1);
            // let every copy still in flight land before the block exits
            if (iss0 > con0) mbar_wait_bounded(&full[0], (iss0 - 1u) & 1u, TC_WAIT);
            if (iss1 > con1) mbar_wait_bounded(&full[1], (iss1 - 1u) & 1u, TC_WAIT);
            mbar_wait_bounded(&wbar, 0, TC_WAIT);
        }
        if (mma_pending) mbar_wait_bounded(&bar, i & 1, TC_WAIT);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::tmem_dealloc(taddr, TCOLS);
}

// --------------------------------------------------------- weight gradient
struct DwArgs {
    const bf16 *in;   // [rows_in][CIN]
    const bf16 *g;    // [rows][COUT], gradient of the conv's pre-activation output
    float *part;      // [gridDim.x][27 * CIN * COUT]
    Lvl lin, lout;
    int64_t rows;
    int *err;
};

constexpr int DW_KV = 32;   // nodes per MMA chunk (GEMM K)

__host__ __device__ constexpr uint32_t pow2_cols(uint32_t c) {
    return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : c <= 256 ? 256 : 512;
}

template <int CIN_, int COUT_>
constexpr size_t dw_smem() {
    return (size_t)((27 + 128 / CIN_ - 1) / (128 / CIN_)) * 128 * DW_KV * 2 + (size_t)COUT_ * DW_KV * 2;
}

template <int CI, int CO, int MODE>
__global__ void __launch_bounds__(128) k_conv_dw_tc(DwArgs a) {
    constexpr int KV = DW_KV;
    constexpr int TPM = 128 / CI;                    // taps per M tile
    constexpr int NMT = (27 + TPM - 1) / TPM;        // M tiles
    constexpr uint32_t MTB = 128u * KV * 2;          // bytes of one M tile
    constexpr uint32_t AB = NMT * MTB;
    constexpr uint32_t BB = (uint32_t)CO * KV * 2;
    constexpr uint32_t TCOLS = pow2_cols(NMT * CO);
    constexpr uint32_t SBO = KV * 16;
    constexpr uint32_t IDESC = tc::idesc_bf16(128, CO);
    static_assert(NMT * CO <= 512, "tensor memory");
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ unsigned long long bar;
    __shared__ uint32_t tslot;
    __shared__ int rb[KV], rx[KV], ry[KV], rz[KV];
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tc::tmem_alloc(&tslot, TCOLS);
    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    for (uint32_t i = tid; i < (AB + BB) / 16; i += 128) reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t taddr = tslot;
    const uint32_t sa = smem_addr(smem), sb = sa + AB;
    unsigned char *pb = smem + AB;
    const int64_t nchunk = (a.rows + KV - 1) / KV;
    uint32_t phase = 0;
    bool ok = true;
    for (int64_t ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
        bool mine = true;
        if (phase > 0) mine = mbar_wait_bounded(&bar, (phase - 1) & 1, TC_WAIT);
        if (!__syncthreads_and(mine)) {
            ok = false;
            break;
        }
        if (tid < KV) {
            const int64_t row = ch * KV + tid;
            if (row < a.rows) {
                int b, x, y, z;
                row_coords(row, a.lout, b, x, y, z);
                rb[tid] = b;
                rx[tid] = x;
                ry[tid] = y;
                rz[tid] = z;
            } else {
                rb[tid] = -1;
            }
        }
        __syncthreads();
        // B = g^T: CO rows x KV nodes
        for (int item = tid; item < KV * (CO / 8); item += 128) {
            const int j = item / (CO / 8), cc = item % (CO / 8);
            uint4 v = make_uint4(0, 0, 0, 0);
            if (rb[j] >= 0) v = __ldg(reinterpret_cast<const uint4 *>(a.g + (ch * KV + j) * CO) + cc);
            const unsigned short *h = reinterpret_cast<const unsigned short *>(&v);
#pragma unroll
            for (int e = 0; e < 8; e++)
                *reinterpret_cast<unsigned short *>(pb + tc::kmaj_off(cc * 8 + e, j, KV)) = h[e];
        }
        // A = gathered input^T: (tap, ci) rows x KV nodes, NMT tiles of 128 rows
        for (int item = tid; item < 27 * KV * (CI / 8); item += 128) {
            const int cc = item % (CI / 8);
            const int rest = item / (CI / 8);
            const int j = rest % KV, t = rest / KV;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (rb[j] >= 0) {
                const int64_t src = gather_src<MODE>(rb[j], rx[j], ry[j], rz[j], t, a.lin);
                if (src >= 0) v = __ldg(reinterpret_cast<const uint4 *>(a.in + src * CI) + cc);
            }
            const int m = t / TPM, r0 = (t % TPM) * CI + cc * 8;
            unsigned char *tileb = smem + m * MTB;
            const unsigned short *h = reinterpret_cast<const unsigned short *>(&v);
#pragma unroll
            for (int e = 0; e < 8; e++)
                *reinterpret_cast<unsigned short *>(tileb + tc::kmaj_off(r0 + e, j, KV)) = h[e];
        }
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            for (int m = 0; m < NMT; m++) {
#pragma unroll
                for (int kk = 0; kk < KV / 16; kk++) {
                    const uint64_t ad = tc::sdesc(sa + m * MTB + kk * 256, 128, SBO);
                    const uint64_t bd = tc::sdesc(sb + kk * 256, 128, SBO);
                    tc::mma_bf16(taddr + m * CO, ad, bd, IDESC, (phase > 0 || kk > 0) ? 1u : 0u);
                }
            }
            tc::mma_commit(&bar);
        }
        phase++;
    }
    bool done = true;
    if (phase > 0) done = mbar_wait_bounded(&bar, (phase - 1) & 1, TC_WAIT);
    if (!__syncthreads_and(done)) ok = false;
    tc::fence_after();
    float *dst = a.part + (size_t)blockIdx.x * (27 * CI * CO);
    for (int m = 0; m < NMT; m++) {
        float v[CO];
#pragma unroll
        for (int c = 0; c < CO / 16; c++)
            tc::tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + m * CO + c * 16, v + c * 16);
        const int t = m * TPM + tid / CI, ci = tid % CI;
        if (t < 27) {
#pragma unroll
            for (int c = 0; c < CO; c++) dst[(t * CI + ci) * CO + c] = (phase > 0 && ok) ? v[c] : 0.0f;
        }
    }
    if (!ok && tid == 0) atomicAdd(a.err, 1);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::tmem_dealloc(taddr, TCOLS);
}

// sum of per-CTA partials (fixed order) into the FP32 gradient, dropping padded input channels
__global__ void k_dw_reduce(const float *part, int nblk, int ci_pad, int ci, int co, float *grad) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 27 * ci * co) return;
    const int c = idx % co, rest = idx / co;
    const int i = rest % ci, t = rest / ci;
    const size_t src = ((size_t)t * ci_pad + i) * co + c;
    const size_t stride = (size_t)27 * ci_pad * co;
    float s = 0.0f;
    for (int b = 0; b < nblk; b++) s += part[b * stride + src];
    grad[idx] = s;
}

// ----------------------------------------------------- CUDA-core layers
// x0 = [in(6), 0 x 10] (host-style FP32 input [rows][6])
__global__ void k_input_f32(const float *in, bf16 *x0, int64_t rows) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const float *q = in + NIN * r;
    float f[8] = {q[0], q[1], q[2], q[3], q[4], q[5], 0, 0};
    uint4 *o = reinterpret_cast<uint4 *>(x0 + r * 16);
    o[0] = pack8(f);
    o[1] = make_uint4(0, 0, 0, 0);
}

// The residual's RMS sqrt(rr / (3 nodec)) (or its inverse), evaluated once
// per block: FP64 division and square root are slow on this part, so no
// thread but the first does them.  Called by every thread before any return.
__device__ __forceinline__ double block_rms(const double *rr, int64_t nodec, bool inverse) {
    __shared__ double s_rms;
    if (threadIdx.x == 0) {
        const double ms = rr[0] / (3.0 * (double)nodec);
        s_rms = ms > 0.0 ? (inverse ? 1.0 / sqrt(ms) : sqrt(ms)) : 0.0;
    }
    __syncthreads();
    return s_rms;
}

// x0 from an FP64 component-major residual, scaled by 1 / sqrt(rr / (3 nodec)),
// and the system's feature channels
__global__ void k_input_r(const double *r, const double *rr, const bf16 *feat, int64_t nodec, int linear, bf16 *x0) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double inv = block_rms(rr, nodec, true);
    if (n >= nodec) return;
    float f[8] = {(float)(r[n] * inv), (float)(r[nodec + n] * inv), (float)(r[2 * nodec + n] * inv),
                  __bfloat162float(feat[3 * n]), __bfloat162float(feat[3 * n + 1]), __bfloat162float(feat[3 * n + 2]),
                  0, 0};
    if (linear)
        for (int c = 0; c < 3; c++) f[3 + c] *= f[c];   // r * phi keeps the map linear in r
    uint4 *o = reinterpret_cast<uint4 *>(x0 + n * 16);
    o[0] = pack8(f);
    o[1] = make_uint4(0, 0, 0, 0);
}

// out = relu(up(coarse) + skip), C channels, one thread per (fine row, 8 channels)
template <int C>
__global__ void k_up_add_relu(const bf16 *coarse, const bf16 *skip, bf16 *out, Lvl lf, Lvl lc, int64_t rows, int act) {
    const int64_t item = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (item >= rows * (C / 8)) return;
    const int64_t row = item / (C / 8);
    const int cc = (int)(item % (C / 8));
    int b, x, y, z;
    row_coords(row, lf, b, x, y, z);
    float acc[8];
    unpack8(__ldg(reinterpret_cast<const uint4 *>(skip + row * C) + cc), acc);
    const int p[3] = {x, y, z};
    int lo[3], nn[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = p[d] >> 1;
        nn[d] = (p[d] & 1) ? 2 : 1;
    }
    for (int k = 0; k < nn[2]; k++)
        for (int j = 0; j < nn[1]; j++)
            for (int i = 0; i < nn[0]; i++) {
                const float w = (nn[0] == 2 ? 0.5f : 1.0f) * (nn[1] == 2 ? 0.5f : 1.0f) * (nn[2] == 2 ? 0.5f : 1.0f);
                const int64_t src =
                    (int64_t)b * lc.v + (lo[0] + i) + (int64_t)lc.n[0] * ((lo[1] + j) + (int64_t)lc.n[1] * (lo[2] + k));
                float f[8];
                unpack8(__ldg(reinterpret_cast<const uint4 *>(coarse + src * C) + cc), f);
#pragma unroll
                for (int e = 0; e < 8; e++) acc[e] += w * f[e];
            }
    if (act) {
#pragma unroll
        for (int e = 0; e < 8; e++) acc[e] = fmaxf(acc[e], 0.0f);
    }
    reinterpret_cast<uint4 *>(out + row * C)[cc] = pack8(acc);
}

// gc = up^T(gf): coarse node I collects fine nodes 2I + d, d in {-1,0,1}^3,
// weight 1 (d = 0) or 1/2 per axis
template <int C>
__global__ void k_restrict(const bf16 *gf, bf16 *gc, Lvl lf, Lvl lc, int64_t rows_c) {
    const int64_t item = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (item >= rows_c * (C / 8)) return;
    const int64_t row = item / (C / 8);
    const int cc = (int)(item % (C / 8));
    int b, x, y, z;
    row_coords(row, lc, b, x, y, z);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dz = -1; dz <= 1; dz++) {
        const int fz = 2 * z + dz;
        if (fz < 0 || fz >= lf.n[2]) continue;
        for (int dy = -1; dy <= 1; dy++) {
            const int fy = 2 * y + dy;
            if (fy < 0 || fy >= lf.n[1]) continue;
            for (int dx = -1; dx <= 1; dx++) {
                const int fx = 2 * x + dx;
                if (fx < 0 || fx >= lf.n[0]) continue;
                const float w = (dx ? 0.5f : 1.0f) * (dy ? 0.5f : 1.0f) * (dz ? 0.5f : 1.0f);
                const int64_t src = (int64_t)b * lf.v + fx + (int64_t)lf.n[0] * (fy + (int64_t)lf.n[1] * fz);
                float f[8];
                unpack8(__ldg(reinterpret_cast<const uint4 *>(gf + src * C) + cc), f);
#pragma unroll
                for (int e = 0; e < 8; e++) acc[e] += w * f[e];
            }
        }
    }
    reinterpret_cast<uint4 *>(gc + row * C)[cc] = pack8(acc);
}

// z = d0 W5 + b5 (FP32 [rows][3])
__global__ void k_output(const bf16 *d0, const float *w5, const float *b5, float *z, int64_t rows) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    float f[16];
    const uint4 *p = reinterpret_cast<const uint4 *>(d0 + r * 16);
    unpack8(p[0], f);
    unpack8(p[1], f + 8);
    for (int c = 0; c < 3; c++) {
        float s = b5 ? b5[c] : 0.0f;
#pragma unroll
        for (int k = 0; k < 16; k++) s += f[k] * w5[k * 3 + c];
        z[3 * r + c] = s;
    }
}

// preconditioner output: z (FP64 component-major) = s * (d0 W5 + b5), zero on
// inactive and boundary rows
__global__ void k_output_precond(const bf16 *d0, const float *w5, const float *b5, const double *rr, int64_t nodec,
                                 const double *adiag, const unsigned char *bcflag, double mtol, const double *r,
                                 double *z) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double s = block_rms(rr, nodec, false);
    if (n >= nodec) return;
    float f[16];
    const uint4 *p = reinterpret_cast<const uint4 *>(d0 + n * 16);
    unpack8(p[0], f);
    unpack8(p[1], f + 8);
    const unsigned char bf = bcflag[n];
    for (int c = 0; c < 3; c++) {
        float o = b5 ? b5[c] : 0.0f;
#pragma unroll
        for (int k = 0; k < 16; k++) o += f[k] * w5[k * 3 + c];
        const int64_t i = c * nodec + n;
        const bool off = (bf & (1 << c)) || !(adiag[i] >= mtol);
        z[i] = off ? 0.0 : (r ? r[i] : 0.0) + s * (double)o;
    }
}

// Linear network: the last prolongation, skip addition and output layer in
// one pass, z = r + s * W5^T (e0 + up(c1)), without storing d0; zero on
// inactive and boundary rows.
template <typename TZ>
__global__ void k_output_up(const bf16 *c1, const bf16 *e0, const float *w5, const double *rr, Lvl lf, Lvl lc,
                            const double *adiag, const unsigned char *bcflag, double mtol, const double *r, TZ *z) {
    __shared__ float sw5[48];
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (threadIdx.x < 48) sw5[threadIdx.x] = w5[threadIdx.x];
    const double s = block_rms(rr, lf.v, false);
    if (n >= lf.v) return;
    const int64_t nodec = lf.v;
    float f[16];
    {
        const uint4 *p = reinterpret_cast<const uint4 *>(e0 + n * 16);
        unpack8(__ldg(p), f);
        unpack8(__ldg(p + 1), f + 8);
    }
    int b_, x, y, zz;
    row_coords(n, lf, b_, x, y, zz);
    const int lo[3] = {x >> 1, y >> 1, zz >> 1}, nn[3] = {(x & 1) ? 2 : 1, (y & 1) ? 2 : 1, (zz & 1) ? 2 : 1};
    const float w = (nn[0] == 2 ? 0.5f : 1.0f) * (nn[1] == 2 ? 0.5f : 1.0f) * (nn[2] == 2 ? 0.5f : 1.0f);
    for (int k = 0; k < nn[2]; k++)
        for (int j = 0; j < nn[1]; j++)
            for (int i = 0; i < nn[0]; i++) {
                const int64_t src = (lo[0] + i) + (int64_t)lc.n[0] * ((lo[1] + j) + (int64_t)lc.n[1] * (lo[2] + k));
                const uint4 *p = reinterpret_cast<const uint4 *>(c1 + src * 16);
                float g[16];
                unpack8(__ldg(p), g);
                unpack8(__ldg(p + 1), g + 8);
#pragma unroll
                for (int e = 0; e < 16; e++) f[e] += w * g[e];
            }
    const unsigned char bf = bcflag[n];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float o = 0.0f;
#pragma unroll
        for (int k = 0; k < 16; k++) o += f[k] * sw5[k * 3 + c];
        const int64_t i = c * nodec + n;
        const bool off = (bf & (1 << c)) || !(adiag[i] >= mtol);
        z[i] = (TZ)(off ? 0.0 : (r ? r[i] : 0.0) + s * (double)o);
    }
}

// adjoint input: gz = the normalized residual (the vector the symmetric
// part is applied to), FP32 [nodec][3]
__global__ void k_adj_seed(const bf16 *x0, float *gz, int64_t nodec) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nodec) return;
    float f[8];
    unpack8(reinterpret_cast<const uint4 *>(x0 + n * 16)[0], f);
    gz[3 * n] = f[0];
    gz[3 * n + 1] = f[1];
    gz[3 * n + 2] = f[2];
}

// gd0 = gz W5^T (linear network: no activation mask)
__global__ void k_output_adj(const float *gz, const float *w5, bf16 *gd0, int64_t rows) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const float g0 = gz[3 * r], g1 = gz[3 * r + 1], g2 = gz[3 * r + 2];
    float o[16];
#pragma unroll
    for (int k = 0; k < 16; k++) o[k] = g0 * w5[k * 3] + g1 * w5[k * 3 + 1] + g2 * w5[k * 3 + 2];
    uint4 *q = reinterpret_cast<uint4 *>(gd0 + r * 16);
    q[0] = pack8(o);
    q[1] = pack8(o + 8);
}

// symmetric preconditioner output: z = r + s/2 (N x + B^T N^T x), x = r / s,
// with N x = d0 W5 and B^T v = v[0:3] + phi * v[3:6] (the input map of the
// linear network); zero on inactive and boundary rows
__global__ void k_output_sym(const bf16 *d0, const bf16 *gx0, const bf16 *feat, const float *w5, const double *rr,
                             int64_t nodec, const double *adiag, const unsigned char *bcflag, double mtol,
                             const double *r, double *z) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double s = block_rms(rr, nodec, false);
    if (n >= nodec) return;
    float f[16], g[8];
    const uint4 *p = reinterpret_cast<const uint4 *>(d0 + n * 16);
    unpack8(p[0], f);
    unpack8(p[1], f + 8);
    unpack8(reinterpret_cast<const uint4 *>(gx0 + n * 16)[0], g);
    const unsigned char bf = bcflag[n];
    for (int c = 0; c < 3; c++) {
        float o = 0.0f;
#pragma unroll
        for (int k = 0; k < 16; k++) o += f[k] * w5[k * 3 + c];
        const float adj = g[c] + __bfloat162float(feat[3 * n + c]) * g[3 + c];
        const int64_t i = c * nodec + n;
        const bool off = (bf & (1 << c)) || !(adiag[i] >= mtol);
        z[i] = off ? 0.0 : r[i] + 0.5 * s * ((double)o + (double)adj);
    }
}

constexpr int RED_THREADS = 256;

// gd0 = (gz W5^T) masked by d0 > 0; per-block partials of dW5 (48) and db5 (3)
__global__ void __launch_bounds__(RED_THREADS) k_output_bwd(const float *gz, const bf16 *d0, const float *w5,
                                                            bf16 *gd0, float *part, int64_t rows, int act) {
    __shared__ float sh[RED_THREADS / 32][51];
    float acc[51];
    for (int i = 0; i < 51; i++) acc[i] = 0.0f;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        float f[16];
        const uint4 *p = reinterpret_cast<const uint4 *>(d0 + r * 16);
        unpack8(p[0], f);
        unpack8(p[1], f + 8);
        const float g0 = gz[3 * r], g1 = gz[3 * r + 1], g2 = gz[3 * r + 2];
        float o[16];
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const float v = g0 * w5[k * 3] + g1 * w5[k * 3 + 1] + g2 * w5[k * 3 + 2];
            o[k] = (!act || f[k] > 0.0f) ? v : 0.0f;
            acc[k * 3] += f[k] * g0;
            acc[k * 3 + 1] += f[k] * g1;
            acc[k * 3 + 2] += f[k] * g2;
        }
        acc[48] += g0;
        acc[49] += g1;
        acc[50] += g2;
        uint4 *q = reinterpret_cast<uint4 *>(gd0 + r * 16);
        q[0] = pack8(o);
        q[1] = pack8(o + 8);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = 0; i < 51; i++) {
        float v = acc[i];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[wid][i] = v;
    }
    __syncthreads();
    if (threadIdx.x < 51) {
        float s = 0.0f;
        for (int w = 0; w < RED_THREADS / 32; w++) s += sh[w][threadIdx.x];
        part[(size_t)blockIdx.x * 51 + threadIdx.x] = s;
    }
}

// per-block channel sums of g [rows][C] (bias gradients)
template <int C>
__global__ void __launch_bounds__(RED_THREADS) k_chan_sum(const bf16 *g, float *part, int64_t rows) {
    __shared__ float sh[RED_THREADS / 32][C];
    float acc[C];
    for (int i = 0; i < C; i++) acc[i] = 0.0f;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        const uint4 *p = reinterpret_cast<const uint4 *>(g + r * C);
#pragma unroll
        for (int c = 0; c < C / 8; c++) {
            float f[8];
            unpack8(p[c], f);
#pragma unroll
            for (int e = 0; e < 8; e++) acc[c * 8 + e] += f[e];
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = 0; i < C; i++) {
        float v = acc[i];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[wid][i] = v;
    }
    __syncthreads();
    if (threadIdx.x < C) {
        float s = 0.0f;
        for (int w = 0; w < RED_THREADS / 32; w++) s += sh[w][threadIdx.x];
        part[(size_t)blockIdx.x * C + threadIdx.x] = s;
    }
}

__global__ void k_part_reduce(const float *part, int nblk, int n, float *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.0f;
    for (int b = 0; b < nblk; b++) s += part[(size_t)b * n + i];
    out[i] = s;
}

// canonical BF16 weight tiles of conv l from the FP32 parameters:
// forward: per tap an N = cout x K = kpad tile of W[t][ci][co];
// transposed (data gradient): per tap an N = cin x K = cout tile.
__global__ void k_wprep(const float *w, int cin, int cout, int kpad, bf16 *fwd, bf16 *trn) {
    const int npad = (cin + 15) / 16 * 16;   // rows of a transposed tile (MMA N, a multiple of 16)
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < 27 * cout * kpad) {
        const int k = idx % kpad, rest = idx / kpad;
        const int n = rest % cout, t = rest / cout;
        const float v = k < cin ? w[((size_t)t * cin + k) * cout + n] : 0.0f;
        const uint32_t off = t * (uint32_t)(cout * kpad * 2) + tc::kmaj_off(n, k, kpad);
        *reinterpret_cast<bf16 *>(reinterpret_cast<unsigned char *>(fwd) + off) = __float2bfloat16_rn(v);
    }
    if (trn && idx < 27 * npad * cout) {
        const int k = idx % cout, rest = idx / cout;
        const int n = rest % npad, t = rest / npad;
        const float v = n < cin ? w[((size_t)t * cin + n) * cout + k] : 0.0f;
        const uint32_t off = t * (uint32_t)(npad * cout * 2) + tc::kmaj_off(n, k, cout);
        *reinterpret_cast<bf16 *>(reinterpret_cast<unsigned char *>(trn) + off) = __float2bfloat16_rn(v);
    }
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// training batch: x0 from stored residuals and their system's features, FP32 targets
__global__ void k_gather_batch(const bf16 *dr, const bf16 *de, const bf16 *df, const int *dsys, const int *idx,
                               int64_t v0, int batch, int linear, int additive, bf16 *x0, float *tgt) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= v0 * batch) return;
    const int b = (int)(r / v0);
    const int64_t n = r - (int64_t)b * v0;
    const int64_t src = (int64_t)idx[b] * v0 + n;
    const int64_t fs = (int64_t)dsys[idx[b]] * v0 + n;
    float f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < 3; c++) {
        f[c] = __bfloat162float(dr[3 * src + c]);
        f[3 + c] = __bfloat162float(df[3 * fs + c]) * (linear ? f[c] : 1.0f);
        tgt[3 * r + c] = __bfloat162float(de[3 * src + c]) - (additive ? f[c] : 0.0f);
    }
    uint4 *o = reinterpret_cast<uint4 *>(x0 + r * 16);
    o[0] = pack8(f);
    o[1] = make_uint4(0, 0, 0, 0);
}

// loss = mean_b |z - t|^2 / |t|^2 ; gz = d loss / d z.  One block per sample.
__global__ void __launch_bounds__(RED_THREADS) k_mse(const float *z, const float *t, float *gz, int64_t v0, int batch,
                                                     float *loss_part) {
    __shared__ float sh[RED_THREADS / 32];
    __shared__ float tot;
    const int b = blockIdx.x;
    const float *zb = z + (size_t)b * v0 * 3, *tb = t + (size_t)b * v0 * 3;
    float *gb = gz + (size_t)b * v0 * 3;
    float s = 0.0f;
    for (int64_t i = threadIdx.x; i < 3 * v0; i += blockDim.x) s += tb[i] * tb[i];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sh[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.0f;
        for (int w = 0; w < RED_THREADS / 32; w++) a += sh[w];
        tot = a > 0.0f ? a : 1.0f;
    }
    __syncthreads();
    const float inv = 1.0f / (tot * (float)batch);
    float l = 0.0f;
    for (int64_t i = threadIdx.x; i < 3 * v0; i += blockDim.x) {
        const float d = zb[i] - tb[i];
        l += d * d;
        gb[i] = 2.0f * d * inv;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    __syncthreads();
    if (lane == 0) sh[wid] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.0f;
        for (int w = 0; w < RED_THREADS / 32; w++) a += sh[w];
        loss_part[b] = a * inv;
    }
}

// training pair: residual and error, both divided by the residual's RMS
__global__ void k_append_pair(const double *r, const double *rr, const double *e, int64_t nodec, bf16 *dr, bf16 *de) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double inv = block_rms(rr, nodec, true);
    if (n >= nodec) return;
    for (int c = 0; c < 3; c++) {
        dr[3 * n + c] = __float2bfloat16_rn((float)(r[c * nodec + n] * inv));
        de[3 * n + c] = __float2bfloat16_rn((float)(e[c * nodec + n] * inv));
    }
}

__global__ void k_set_int(int *p, int v) { *p = v; }

// feature channels of a system: phi (FP64 component-major) -> bf16 [nodec][3]
__global__ void k_feature(const double *phi, int64_t nodec, bf16 *feat) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nodec) return;
    for (int c = 0; c < 3; c++) feat[3 * n + c] = __float2bfloat16_rn((float)phi[c * nodec + n]);
}

}  // namespace nn
}  // namespace mpm

// ------------------------------------------------------------- network object
struct mpm_nn {
    nn::Lvl L[3];
    int max_batch = 1;
    int nsm = 148;
    float *p = nullptr, *g = nullptr, *am = nullptr, *av = nullptr;
    bf16 *wf[NCONV] = {}, *wt[NCONV] = {};
    bf16 *x0 = nullptr, *e0 = nullptr, *e1 = nullptr, *e2 = nullptr, *c2 = nullptr, *d1 = nullptr, *c1 = nullptr,
         *d0 = nullptr;
    bf16 *gd0 = nullptr, *ge0 = nullptr, *gc1 = nullptr, *gd1 = nullptr, *ge1 = nullptr, *gc2 = nullptr,
         *ge2 = nullptr;
    float *z = nullptr, *gz = nullptr, *tgt = nullptr;
    float *part = nullptr;
    size_t part_cap = 0;
    float *loss = nullptr;
    int *idx = nullptr;
    int *err = nullptr;
    bool weights_dirty = true;
    int linear = 1;     // 1: no activations and no biases (a linear operator of the input)
    int additive = 1;   // 1: preconditioner r + net(r), the network trained on (error - residual)
    int symmetric = 0;  // 1 (linear, additive): apply r + (N + N^T) r / 2
    int halo = 1;       // forward convolutions on halo tiles (k_conv_halo); 0: per-tap gathers (k_conv_tc)
    bf16 *gx0 = nullptr;   // adjoint result at the input [v0][16]
    int64_t adam_step = 0;
    bf16 *data_r = nullptr, *data_e = nullptr;
    int64_t ndata = 0, data_cap = 0;
    bf16 *feat = nullptr;        // feature channels of the system being solved [v0][3]
    bf16 *data_f = nullptr;      // feature channels of each harvested system [max_systems][v0][3]
    int *data_sys = nullptr;     // system of each stored pair
    int nsys = 0, sys_cap = 0;
    int64_t *d_ndata = nullptr;
    cudaStream_t stream = nullptr;
};

namespace {

using namespace mpm::nn;

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda)
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        cudaGetLastError();
    }
    return fn;
}

// The per-chunk tensor maps of a channels-last BF16 activation [batch][z][y][x][K]
// for the halo copies of k_conv_halo: dims (8 channels, x, y, z, sample),
// box (8, S1 ? 10 : 18, S1 ? 18 : 33, 3, 1), x traversal stride 1 (S1) or 2 (S2).
template <int K, int MODE>
bool make_halo_maps(const bf16 *in, const Lvl &L, int batch, HaloMaps &m) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dims[5] = {8, (cuuint64_t)L.n[0], (cuuint64_t)L.n[1], (cuuint64_t)L.n[2], (cuuint64_t)batch};
    const cuuint64_t es = (cuuint64_t)K * 2;
    const cuuint64_t strides[4] = {es, es * L.n[0], es * L.n[0] * L.n[1], es * (cuuint64_t)L.v};
    // S2: 9 elements at stride 2 (the driver loads ceil(box / stride) elements)
    const cuuint32_t box[5] = {8, MODE == S1 ? 10u : 18u, (cuuint32_t)Halo<MODE>::HY, 3, 1};
    const cuuint32_t estr[5] = {1, MODE == S1 ? 1u : 2u, 1, 1, 1};
    for (int kc = 0; kc < K / 8; kc++) {
        CUresult r = enc(&m.m[kc], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(in) + kc * 8, dims, strides,
                         box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return false;
    }
    return true;
}

template <int K, int N, int MODE>
cudaError_t launch_conv_halo(mpm_nn *net, cudaStream_t st, const ConvArgs &a) {
    constexpr size_t smem = halo_smem<K, N, MODE>();
    static_assert(smem <= 227u * 1024, "shared memory");
    HaloMaps maps;
    memset(&maps, 0, sizeof(maps));
    if (!make_halo_maps<K, MODE>(a.in, a.lin, (int)(a.rows / a.lout.v), maps)) return cudaErrorNotSupported;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_conv_halo<K, N, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int64_t ntile = (int64_t)(a.rows / a.lout.v) * ((a.lout.n[0] + 7) / 8) * ((a.lout.n[1] + 15) / 16) *
                          a.lout.n[2];
    const int per_sm = std::max<int>(1, std::min<int>(4, (int)(225000 / (smem + 1024))));
    const int grid = (int)std::min<int64_t>(ntile, (int64_t)net->nsm * per_sm);
    if (grid <= 0) return cudaSuccess;
    k_conv_halo<K, N, MODE><<<grid, 128, smem, st>>>(a, maps);
    return cudaGetLastError();
}

template <int K, int N, int MODE>
cudaError_t launch_conv(mpm_nn *net, cudaStream_t st, const bf16 *in, bf16 *out, const bf16 *w, const float *bias,
                        const bf16 *add, const bf16 *mask, int relu, const Lvl &lin, const Lvl &lout, int batch) {
    constexpr size_t smem = conv_smem<K, N>();
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_conv_tc<K, N, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    ConvArgs a;
    a.in = in;
    a.out = out;
    a.w = w;
    a.bias = bias;
    a.add = add;
    a.mask = mask;
    a.relu = relu;
    a.lin = lin;
    a.lout = lout;
    a.rows = (int64_t)batch * lout.v;
    a.err = net->err;
    if constexpr (MODE == S1 || MODE == S2) {
        if (net->halo) return launch_conv_halo<K, N, MODE>(net, st, a);
    }
    const int64_t ntile = (a.rows + 127) / 128;
    const int per_sm = std::max<int>(1, std::min<int>(4, (int)(220000 / smem)));
    const int grid = (int)std::min<int64_t>(ntile, (int64_t)net->nsm * per_sm);
    k_conv_tc<K, N, MODE><<<grid, 128, smem, st>>>(a);
    return cudaGetLastError();
}

template <int CI, int CO, int MODE>
cudaError_t launch_dw(mpm_nn *net, cudaStream_t st, const bf16 *in, const bf16 *g, const Lvl &lin, const Lvl &lout,
                      int batch, int ci_real, float *grad) {
    constexpr size_t smem = dw_smem<CI, CO>();
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_conv_dw_tc<CI, CO, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    DwArgs a;
    a.in = in;
    a.g = g;
    a.lin = lin;
    a.lout = lout;
    a.rows = (int64_t)batch * lout.v;
    a.err = net->err;
    const int64_t nchunk = (a.rows + DW_KV - 1) / DW_KV;
    int grid = (int)std::min<int64_t>(nchunk, (int64_t)net->nsm);
    const size_t per = (size_t)27 * CI * CO;
    if ((size_t)grid * per > net->part_cap) grid = (int)(net->part_cap / per);
    a.part = net->part;
    k_conv_dw_tc<CI, CO, MODE><<<grid, 128, smem, st>>>(a);
    const int n = 27 * ci_real * CO;
    k_dw_reduce<<<(n + 255) / 256, 256, 0, st>>>(net->part, grid, CI, ci_real, CO, grad);
    return cudaGetLastError();
}

template <int C>
void launch_chan_sum(mpm_nn *net, cudaStream_t st, const bf16 *g, int64_t rows, float *out) {
    const int nblk = (int)std::min<int64_t>((rows + RED_THREADS - 1) / RED_THREADS, 2 * (int64_t)net->nsm);
    k_chan_sum<C><<<nblk, RED_THREADS, 0, st>>>(g, net->part, rows);
    k_part_reduce<<<1, 64, 0, st>>>(net->part, nblk, C, out);
}

int blocks(int64_t n, int t = 256) { return (int)((n + t - 1) / t); }

cudaError_t prep_weights(mpm_nn *net, cudaStream_t st) {
    if (!net->weights_dirty) return cudaSuccess;
    for (int l = 0; l < NCONV; l++) {
        const int n = 27 * COUT[l] * std::max(KPAD[l], CIN[l]);
        k_wprep<<<blocks(n), 256, 0, st>>>(net->p + w_offset(l), CIN[l], COUT[l], KPAD[l], net->wf[l], net->wt[l]);
    }
    net->weights_dirty = false;
    return cudaGetLastError();
}

// forward of `batch` samples whose x0 is already in place
cudaError_t forward(mpm_nn *net, cudaStream_t st, int batch, bool make_d0 = true) {
    cudaError_t e = prep_weights(net, st);
    if (e != cudaSuccess) return e;
    const Lvl &L0 = net->L[0], &L1 = net->L[1], &L2 = net->L[2];
    const float *P = net->p;
    const int act = net->linear ? 0 : 1;
    auto bias = [&](int l) -> const float * { return net->linear ? nullptr : P + b_offset(l); };
    if ((e = launch_conv<16, 16, S1>(net, st, net->x0, net->e0, net->wf[0], bias(0), nullptr, nullptr, act, L0, L0,
                                     batch)) != cudaSuccess)
        return e;
    if ((e = launch_conv<16, 32, S2>(net, st, net->e0, net->e1, net->wf[1], bias(1), nullptr, nullptr, act, L0, L1,
                                     batch)) != cudaSuccess)
        return e;
    if ((e = launch_conv<32, 64, S2>(net, st, net->e1, net->e2, net->wf[2], bias(2), nullptr, nullptr, act, L1, L2,
                                     batch)) != cudaSuccess)
        return e;
    if ((e = launch_conv<64, 32, S1>(net, st, net->e2, net->c2, net->wf[3], bias(3), nullptr, nullptr, 0, L2, L2,
                                     batch)) != cudaSuccess)
        return e;
    const int64_t r1 = (int64_t)batch * L1.v, r0 = (int64_t)batch * L0.v;
    k_up_add_relu<32><<<blocks(r1 * 4), 256, 0, st>>>(net->c2, net->e1, net->d1, L1, L2, r1, act);
    if ((e = launch_conv<32, 16, S1>(net, st, net->d1, net->c1, net->wf[4], bias(4), nullptr, nullptr, 0, L1, L1,
                                     batch)) != cudaSuccess)
        return e;
    if (make_d0) k_up_add_relu<16><<<blocks(r0 * 2), 256, 0, st>>>(net->c1, net->e0, net->d0, L0, L1, r0, act);
    return cudaGetLastError();
}

// backward from gz (FP32 [rows0][3]) into net->g
cudaError_t backward(mpm_nn *net, cudaStream_t st, int batch) {
    const Lvl &L0 = net->L[0], &L1 = net->L[1], &L2 = net->L[2];
    const int64_t r0 = (int64_t)batch * L0.v, r1 = (int64_t)batch * L1.v, r2 = (int64_t)batch * L2.v;
    float *G = net->g;
    cudaError_t e;
    {
        const int nblk = (int)std::min<int64_t>(blocks(r0, RED_THREADS), 2 * (int64_t)net->nsm);
        k_output_bwd<<<nblk, RED_THREADS, 0, st>>>(net->gz, net->d0, net->p + w5_offset(), net->gd0, net->part, r0,
                                                   net->linear ? 0 : 1);
        k_part_reduce<<<1, 64, 0, st>>>(net->part, nblk, 51, G + w5_offset());
    }
    // c1 -> d0 through up: gc1 = up^T(gd0)
    k_restrict<16><<<blocks(r1 * 2), 256, 0, st>>>(net->gd0, net->gc1, L0, L1, r1);
    const bool lin = net->linear != 0;
    if (!lin) launch_chan_sum<16>(net, st, net->gc1, r1, G + b_offset(4));
    if ((e = launch_dw<32, 16, S1>(net, st, net->d1, net->gc1, L1, L1, batch, 32, G + w_offset(4))) != cudaSuccess)
        return e;
    // gd1 = conv4^T(gc1) masked by d1
    if ((e = launch_conv<16, 32, S1T>(net, st, net->gc1, net->gd1, net->wt[4], nullptr, nullptr, lin ? nullptr : net->d1, 0, L1, L1,
                                      batch)) != cudaSuccess)
        return e;
    k_restrict<32><<<blocks(r2 * 4), 256, 0, st>>>(net->gd1, net->gc2, L1, L2, r2);
    if (!lin) launch_chan_sum<32>(net, st, net->gc2, r2, G + b_offset(3));
    if ((e = launch_dw<64, 32, S1>(net, st, net->e2, net->gc2, L2, L2, batch, 64, G + w_offset(3))) != cudaSuccess)
        return e;
    // ge2 = conv3^T(gc2) masked by e2
    if ((e = launch_conv<32, 64, S1T>(net, st, net->gc2, net->ge2, net->wt[3], nullptr, nullptr, lin ? nullptr : net->e2, 0, L2, L2,
                                      batch)) != cudaSuccess)
        return e;
    if (!lin) launch_chan_sum<64>(net, st, net->ge2, r2, G + b_offset(2));
    if ((e = launch_dw<32, 64, S2>(net, st, net->e1, net->ge2, L1, L2, batch, 32, G + w_offset(2))) != cudaSuccess)
        return e;
    // ge1 = (conv2^T(ge2) + gd1) masked by e1
    if ((e = launch_conv<64, 32, S2T>(net, st, net->ge2, net->ge1, net->wt[2], nullptr, net->gd1, lin ? nullptr : net->e1, 0, L2, L1,
                                      batch)) != cudaSuccess)
        return e;
    if (!lin) launch_chan_sum<32>(net, st, net->ge1, r1, G + b_offset(1));
    if ((e = launch_dw<16, 32, S2>(net, st, net->e0, net->ge1, L0, L1, batch, 16, G + w_offset(1))) != cudaSuccess)
        return e;
    // ge0 = (conv1^T(ge1) + gd0) masked by e0
    if ((e = launch_conv<32, 16, S2T>(net, st, net->ge1, net->ge0, net->wt[1], nullptr, net->gd0, lin ? nullptr : net->e0, 0, L1, L0,
                                      batch)) != cudaSuccess)
        return e;
    if (!lin) launch_chan_sum<16>(net, st, net->ge0, r0, G + b_offset(0));
    if (lin) {   // biases are not used: their gradients are zero
        for (int l = 0; l < NCONV; l++) cudaMemsetAsync(G + b_offset(l), 0, sizeof(float) * COUT[l], st);
        cudaMemsetAsync(G + b5_offset(), 0, sizeof(float) * 3, st);
    }
    if ((e = launch_dw<16, 16, S1>(net, st, net->x0, net->ge0, L0, L0, batch, NIN, G + w_offset(0))) != cudaSuccess)
        return e;
    return cudaGetLastError();
}

// N^T applied to net->gz (linear network): the data-gradient chain of
// backward() without weight gradients, down to the input x0 (net->gx0)
cudaError_t adjoint(mpm_nn *net, cudaStream_t st) {
    const Lvl &L0 = net->L[0], &L1 = net->L[1], &L2 = net->L[2];
    const int64_t r0 = L0.v, r1 = L1.v, r2 = L2.v;
    cudaError_t e;
    k_output_adj<<<blocks(r0), 256, 0, st>>>(net->gz, net->p + w5_offset(), net->gd0, r0);
    k_restrict<16><<<blocks(r1 * 2), 256, 0, st>>>(net->gd0, net->gc1, L0, L1, r1);
    if ((e = launch_conv<16, 32, S1T>(net, st, net->gc1, net->gd1, net->wt[4], nullptr, nullptr, nullptr, 0, L1, L1,
                                      1)) != cudaSuccess)
        return e;
    k_restrict<32><<<blocks(r2 * 4), 256, 0, st>>>(net->gd1, net->gc2, L1, L2, r2);
    if ((e = launch_conv<32, 64, S1T>(net, st, net->gc2, net->ge2, net->wt[3], nullptr, nullptr, nullptr, 0, L2, L2,
                                      1)) != cudaSuccess)
        return e;
    if ((e = launch_conv<64, 32, S2T>(net, st, net->ge2, net->ge1, net->wt[2], nullptr, net->gd1, nullptr, 0, L2, L1,
                                      1)) != cudaSuccess)
        return e;
    if ((e = launch_conv<32, 16, S2T>(net, st, net->ge1, net->ge0, net->wt[1], nullptr, net->gd0, nullptr, 0, L1, L0,
                                      1)) != cudaSuccess)
        return e;
    if ((e = launch_conv<16, 16, S1T>(net, st, net->ge0, net->gx0, net->wt[0], nullptr, nullptr, nullptr, 0, L0, L0,
                                      1)) != cudaSuccess)
        return e;
    return cudaGetLastError();
}

mpm_status read_err(mpm_nn *net) {
    int h = 0;
    CKN(cudaMemcpy(&h, net->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        CKN(cudaMemset(net->err, 0, sizeof(int)));
        return MPM_ERR_DEVICE_TIMEOUT;
    }
    return MPM_OK;
}

void net_free(mpm_nn *n) {
    void *ptrs[] = {n->p,   n->g,   n->am,  n->av,  n->x0,  n->e0,  n->e1,  n->e2,     n->c2,     n->d1,
                    n->c1,  n->d0,  n->gd0, n->ge0, n->gc1, n->gd1, n->ge1, n->gc2,    n->ge2,    n->z,
                    n->gz,  n->tgt, n->part, n->loss, n->idx, n->err, n->data_r, n->data_e, n->d_ndata,
                    n->feat, n->data_f, n->data_sys, n->gx0};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int l = 0; l < NCONV; l++) {
        if (n->wf[l]) cudaFree(n->wf[l]);
        if (n->wt[l]) cudaFree(n->wt[l]);
    }
}

// splitmix64 + Box-Muller: deterministic parameter initialisation
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    }
};

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

int64_t mpm_nn_num_params(void) { return param_count(); }

mpm_status mpm_nn_create(const int nodes[3], int max_batch, int64_t max_pairs, mpm_nn **out) {
    if (!nodes || !out || max_batch < 1 || max_pairs < 0) return MPM_ERR_BAD_ARG;
    for (int d = 0; d < 3; d++)
        if (nodes[d] < 3) return MPM_ERR_BAD_ARG;
    // row indices of a batch are 32-bit on the device
    if ((int64_t)nodes[0] * nodes[1] * nodes[2] * (int64_t)max_batch >= ((int64_t)1 << 31)) return MPM_ERR_BAD_ARG;
    mpm_nn *n = new (std::nothrow) mpm_nn();
    if (!n) return MPM_ERR_OOM;
    for (int d = 0; d < 3; d++) {
        n->L[0].n[d] = nodes[d];
        n->L[1].n[d] = nodes[d] / 2 + 1;
        n->L[2].n[d] = n->L[1].n[d] / 2 + 1;
    }
    for (int l = 0; l < 3; l++) n->L[l].v = (int64_t)n->L[l].n[0] * n->L[l].n[1] * n->L[l].n[2];
    n->max_batch = max_batch;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n->nsm, cudaDevAttrMultiProcessorCount, dev);
    if (const char *g = getenv("MPM_GB300_CONV_GATHER")) n->halo = atoi(g) ? 0 : 1;
    const int64_t P = param_count();
    const int64_t B = max_batch, v0 = n->L[0].v, v1 = n->L[1].v, v2 = n->L[2].v;
    auto fail = [&](cudaError_t e) {
        fprintf(stderr, "mpm_gb300 (nn): allocation failed: %s\n", cudaGetErrorString(e));
        net_free(n);
        delete n;
        return e == cudaErrorMemoryAllocation ? MPM_ERR_OOM : MPM_ERR_CUDA;
    };
    cudaError_t e;
#define NN_ALLOC(ptr, bytes)                                       \
    do {                                                           \
        if ((e = cudaMalloc((void **)&(ptr), (bytes))) != cudaSuccess) return fail(e); \
    } while (0)
    NN_ALLOC(n->p, P * 4);
    NN_ALLOC(n->g, P * 4);
    NN_ALLOC(n->am, P * 4);
    NN_ALLOC(n->av, P * 4);
    for (int l = 0; l < NCONV; l++) {
        NN_ALLOC(n->wf[l], (size_t)27 * COUT[l] * KPAD[l] * 2);
        NN_ALLOC(n->wt[l], (size_t)27 * ((CIN[l] + 15) / 16 * 16) * COUT[l] * 2);
    }
    NN_ALLOC(n->x0, B * v0 * 16 * 2);
    NN_ALLOC(n->e0, B * v0 * 16 * 2);
    NN_ALLOC(n->d0, B * v0 * 16 * 2);
    NN_ALLOC(n->gd0, B * v0 * 16 * 2);
    NN_ALLOC(n->ge0, B * v0 * 16 * 2);
    NN_ALLOC(n->e1, B * v1 * 32 * 2);
    NN_ALLOC(n->d1, B * v1 * 32 * 2);
    NN_ALLOC(n->c1, B * v1 * 16 * 2);
    NN_ALLOC(n->gc1, B * v1 * 16 * 2);
    NN_ALLOC(n->gd1, B * v1 * 32 * 2);
    NN_ALLOC(n->ge1, B * v1 * 32 * 2);
    NN_ALLOC(n->e2, B * v2 * 64 * 2);
    NN_ALLOC(n->c2, B * v2 * 32 * 2);
    NN_ALLOC(n->gc2, B * v2 * 32 * 2);
    NN_ALLOC(n->ge2, B * v2 * 64 * 2);
    NN_ALLOC(n->z, B * v0 * 3 * 4);
    NN_ALLOC(n->gz, B * v0 * 3 * 4);
    NN_ALLOC(n->tgt, B * v0 * NIN * 4);
    n->part_cap = (size_t)n->nsm * 27 * 64 * 32;   // largest weight-gradient partials
    NN_ALLOC(n->part, n->part_cap * 4);
    NN_ALLOC(n->loss, (size_t)B * 4);
    NN_ALLOC(n->idx, (size_t)B * 4);
    NN_ALLOC(n->err, sizeof(int));
    NN_ALLOC(n->d_ndata, sizeof(int64_t));
    NN_ALLOC(n->feat, (size_t)v0 * 3 * 2);
    NN_ALLOC(n->gx0, (size_t)v0 * 16 * 2);
    if (max_pairs > 0) {
        NN_ALLOC(n->data_r, (size_t)max_pairs * v0 * 3 * 2);
        NN_ALLOC(n->data_e, (size_t)max_pairs * v0 * 3 * 2);
        NN_ALLOC(n->data_sys, (size_t)max_pairs * sizeof(int));
        n->sys_cap = (int)std::min<int64_t>(max_pairs, 512);
        NN_ALLOC(n->data_f, (size_t)n->sys_cap * v0 * 3 * 2);
    }
#undef NN_ALLOC
    n->data_cap = max_pairs;
    cudaMemset(n->p, 0, P * 4);
    cudaMemset(n->am, 0, P * 4);
    cudaMemset(n->av, 0, P * 4);
    cudaMemset(n->err, 0, sizeof(int));
    cudaMemset(n->feat, 0, (size_t)v0 * 3 * 2);
    *out = n;
    return MPM_OK;
}

mpm_status mpm_nn_destroy(mpm_nn *net) {
    if (!net) return MPM_ERR_BAD_ARG;
    cudaDeviceSynchronize();
    net_free(net);
    delete net;
    return MPM_OK;
}

mpm_status mpm_nn_set_linear(mpm_nn *net, int linear) {
    if (!net) return MPM_ERR_BAD_ARG;
    net->linear = linear ? 1 : 0;
    return MPM_OK;
}

mpm_status mpm_nn_set_symmetric(mpm_nn *net, int symmetric) {
    if (!net) return MPM_ERR_BAD_ARG;
    net->symmetric = symmetric ? 1 : 0;
    return MPM_OK;
}

mpm_status mpm_nn_set_additive(mpm_nn *net, int additive) {
    if (!net) return MPM_ERR_BAD_ARG;
    net->additive = additive ? 1 : 0;
    return MPM_OK;
}

mpm_status mpm_nn_set_stream(mpm_nn *net, void *stream) {
    if (!net) return MPM_ERR_BAD_ARG;
    net->stream = (cudaStream_t)stream;
    return MPM_OK;
}

mpm_status mpm_nn_init_params(mpm_nn *net, uint64_t seed) {
    if (!net) return MPM_ERR_BAD_ARG;
    std::vector<float> h(param_count(), 0.0f);
    Rng rng{seed};
    for (int l = 0; l < NCONV; l++) {
        const double sd = sqrt(2.0 / (27.0 * CIN[l]));
        float *w = h.data() + w_offset(l);
        for (int64_t i = 0; i < 27LL * CIN[l] * COUT[l]; i++) w[i] = (float)(sd * rng.normal());
    }
    const double sd5 = sqrt(1.0 / 16.0);
    for (int i = 0; i < 48; i++) h[w5_offset() + i] = (float)(sd5 * rng.normal());
    CKN(cudaMemcpy(net->p, h.data(), h.size() * 4, cudaMemcpyHostToDevice));
    CKN(cudaMemset(net->am, 0, h.size() * 4));
    CKN(cudaMemset(net->av, 0, h.size() * 4));
    net->adam_step = 0;
    net->weights_dirty = true;
    return MPM_OK;
}

mpm_status mpm_nn_set_params(mpm_nn *net, const float *params) {
    if (!net || !params) return MPM_ERR_BAD_ARG;
    CKN(cudaMemcpy(net->p, params, param_count() * 4, cudaMemcpyHostToDevice));
    net->weights_dirty = true;
    return MPM_OK;
}

mpm_status mpm_nn_get_params(mpm_nn *net, float *params) {
    if (!net || !params) return MPM_ERR_BAD_ARG;
    CKN(cudaStreamSynchronize(net->stream));
    CKN(cudaMemcpy(params, net->p, param_count() * 4, cudaMemcpyDeviceToHost));
    return MPM_OK;
}

mpm_status mpm_nn_forward(mpm_nn *net, int batch, const float *in, float *out) {
    if (!net || !in || !out || batch < 1 || batch > net->max_batch) return MPM_ERR_BAD_ARG;
    cudaStream_t st = net->stream;
    const int64_t r0 = (int64_t)batch * net->L[0].v;
    CKN(cudaMemcpyAsync(net->tgt, in, r0 * NIN * 4, cudaMemcpyHostToDevice, st));
    k_input_f32<<<blocks(r0), 256, 0, st>>>(net->tgt, net->x0, r0);
    CKN(forward(net, st, batch));
    k_output<<<blocks(r0), 256, 0, st>>>(net->d0, net->p + w5_offset(), net->linear ? nullptr : net->p + b5_offset(), net->z, r0);
    CKN(cudaGetLastError());
    CKN(cudaMemcpyAsync(out, net->z, r0 * 3 * 4, cudaMemcpyDeviceToHost, st));
    CKN(cudaStreamSynchronize(st));
    return read_err(net);
}

mpm_status mpm_nn_backward(mpm_nn *net, int batch, const float *in, const float *gout, float *grad) {
    if (!net || !in || !gout || !grad || batch < 1 || batch > net->max_batch) return MPM_ERR_BAD_ARG;
    cudaStream_t st = net->stream;
    const int64_t r0 = (int64_t)batch * net->L[0].v;
    CKN(cudaMemcpyAsync(net->tgt, in, r0 * NIN * 4, cudaMemcpyHostToDevice, st));
    CKN(cudaMemcpyAsync(net->gz, gout, r0 * 3 * 4, cudaMemcpyHostToDevice, st));
    k_input_f32<<<blocks(r0), 256, 0, st>>>(net->tgt, net->x0, r0);
    CKN(forward(net, st, batch));
    CKN(backward(net, st, batch));
    CKN(cudaMemcpyAsync(grad, net->g, param_count() * 4, cudaMemcpyDeviceToHost, st));
    CKN(cudaStreamSynchronize(st));
    return read_err(net);
}

mpm_status mpm_nn_num_pairs(mpm_nn *net, int64_t *n) {
    if (!net || !n) return MPM_ERR_BAD_ARG;
    *n = net->ndata;
    return MPM_OK;
}

mpm_status mpm_nn_train(mpm_nn *net, int epochs, int batch, double lr, uint64_t seed, float *epoch_loss) {
    if (!net || epochs < 1 || batch < 1 || batch > net->max_batch || !(lr > 0.0)) return MPM_ERR_BAD_ARG;
    if (net->ndata < batch) return MPM_ERR_STATE;
    cudaStream_t st = net->stream;
    const int64_t v0 = net->L[0].v, r0 = (int64_t)batch * v0;
    const int64_t P = param_count();
    const int64_t nb = net->ndata / batch;
    std::vector<int> perm(net->ndata);
    std::vector<float> lbuf(batch);
    Rng rng{seed};
    const float b1 = 0.9f, b2 = 0.999f;
    for (int ep = 0; ep < epochs; ep++) {
        for (int64_t i = 0; i < net->ndata; i++) perm[i] = (int)i;
        for (int64_t i = net->ndata - 1; i > 0; i--) std::swap(perm[i], perm[rng.next() % (uint64_t)(i + 1)]);
        double lsum = 0.0;
        for (int64_t bi = 0; bi < nb; bi++) {
            CKN(cudaMemcpyAsync(net->idx, perm.data() + bi * batch, batch * 4, cudaMemcpyHostToDevice, st));
            k_gather_batch<<<blocks(r0), 256, 0, st>>>(net->data_r, net->data_e, net->data_f, net->data_sys,
                                                       net->idx, v0, batch, net->linear, net->additive, net->x0,
                                                       net->tgt);
            CKN(forward(net, st, batch));
            k_output<<<blocks(r0), 256, 0, st>>>(net->d0, net->p + w5_offset(), net->linear ? nullptr : net->p + b5_offset(), net->z, r0);
            k_mse<<<batch, RED_THREADS, 0, st>>>(net->z, net->tgt, net->gz, v0, batch, net->loss);
            CKN(backward(net, st, batch));
            net->adam_step++;
            const float c1 = 1.0f - powf(b1, (float)net->adam_step), c2 = 1.0f - powf(b2, (float)net->adam_step);
            // cosine decay of the step size over the whole call
            const double prog = (double)(ep * nb + bi) / (double)(epochs * nb);
            const float lr_t = (float)(lr * 0.5 * (1.0 + cos(3.141592653589793 * prog)));
            k_adam<<<blocks(P), 256, 0, st>>>(net->p, net->g, net->am, net->av, P, lr_t, b1, b2, 1e-8f, c1, c2);
            net->weights_dirty = true;
            CKN(cudaMemcpyAsync(lbuf.data(), net->loss, batch * 4, cudaMemcpyDeviceToHost, st));
            CKN(cudaStreamSynchronize(st));
            for (int b = 0; b < batch; b++) lsum += lbuf[b];
        }
        if (epoch_loss) epoch_loss[ep] = (float)(lsum / (double)nb);
    }
    CKN(cudaStreamSynchronize(st));
    return read_err(net);
}

}  // extern "C"

// ------------------------------------------------------- solver-side hooks
int mpm_nn_grid_matches(const mpm_nn *net, const int nodes[3]) {
    return net && net->L[0].n[0] == nodes[0] && net->L[0].n[1] == nodes[1] && net->L[0].n[2] == nodes[2];
}

mpm_status mpm_nn_apply_precond(mpm_nn *net, cudaStream_t st, const double *r, const double *rr, const double *adiag,
                                const unsigned char *bcflag, double mtol, double *z) {
    const int64_t nodec = net->L[0].v;
    k_input_r<<<blocks(nodec), 256, 0, st>>>(r, rr, net->feat, nodec, net->linear, net->x0);
    if (net->linear && !net->symmetric) {
        CKN(forward(net, st, 1, false));
        k_output_up<double><<<blocks(nodec), 256, 0, st>>>(net->c1, net->e0, net->p + w5_offset(), rr, net->L[0],
                                                           net->L[1], adiag, bcflag, mtol,
                                                           net->additive ? r : nullptr, z);
        CKN(cudaGetLastError());
        return MPM_OK;
    }
    CKN(forward(net, st, 1));
    if (net->symmetric && net->linear && net->additive) {
        k_adj_seed<<<blocks(nodec), 256, 0, st>>>(net->x0, net->gz, nodec);
        CKN(adjoint(net, st));
        k_output_sym<<<blocks(nodec), 256, 0, st>>>(net->d0, net->gx0, net->feat, net->p + w5_offset(), rr, nodec,
                                                   adiag, bcflag, mtol, r, z);
        CKN(cudaGetLastError());
        return MPM_OK;
    }
    k_output_precond<<<blocks(nodec), 256, 0, st>>>(net->d0, net->p + w5_offset(),
                                                   net->linear ? nullptr : net->p + b5_offset(), rr, nodec,
                                                   adiag, bcflag, mtol, net->additive ? r : nullptr, z);
    CKN(cudaGetLastError());
    return MPM_OK;
}

int mpm_nn_fp32_output(const mpm_nn *net) { return net && net->linear && !net->symmetric; }

mpm_status mpm_nn_apply_precond_f32(mpm_nn *net, cudaStream_t st, const double *r, const double *rr,
                                    const double *adiag, const unsigned char *bcflag, double mtol, float *z) {
    if (!mpm_nn_fp32_output(net)) return MPM_ERR_UNSUPPORTED;
    const int64_t nodec = net->L[0].v;
    k_input_r<<<blocks(nodec), 256, 0, st>>>(r, rr, net->feat, nodec, net->linear, net->x0);
    CKN(forward(net, st, 1, false));
    k_output_up<float><<<blocks(nodec), 256, 0, st>>>(net->c1, net->e0, net->p + w5_offset(), rr, net->L[0],
                                                      net->L[1], adiag, bcflag, mtol, net->additive ? r : nullptr, z);
    CKN(cudaGetLastError());
    return MPM_OK;
}

mpm_status mpm_nn_set_feature(mpm_nn *net, cudaStream_t st, const double *phi) {
    const int64_t nodec = net->L[0].v;
    k_feature<<<blocks(nodec), 256, 0, st>>>(phi, nodec, net->feat);
    CKN(cudaGetLastError());
    return MPM_OK;
}

mpm_status mpm_nn_begin_system(mpm_nn *net, cudaStream_t st, const double *phi) {
    if (net->nsys >= net->sys_cap) return MPM_ERR_BAD_ARG;
    const int64_t nodec = net->L[0].v;
    k_feature<<<blocks(nodec), 256, 0, st>>>(phi, nodec, net->data_f + (size_t)net->nsys * nodec * 3);
    net->nsys++;
    CKN(cudaGetLastError());
    return MPM_OK;
}

mpm_status mpm_nn_append_pair(mpm_nn *net, cudaStream_t st, const double *r, const double *rr, const double *e) {
    if (net->ndata >= net->data_cap || net->nsys == 0) return MPM_OK;
    k_set_int<<<1, 1, 0, st>>>(net->data_sys + net->ndata, net->nsys - 1);
    const int64_t nodec = net->L[0].v;
    k_append_pair<<<blocks(nodec), 256, 0, st>>>(r, rr, e, nodec, net->data_r + net->ndata * nodec * 3,
                                                net->data_e + net->ndata * nodec * 3);
    net->ndata++;
    CKN(cudaGetLastError());
    return MPM_OK;
}
