// P2G scatter that allocates no device memory: mpm_gpu_p2g_noalloc.
//
// Who needs it: a caller that embeds this library inside a host program that
// owns every device allocation (a coupling framework with its own memory
// pool, or a solver that must not trigger the implicit device-wide
// synchronisation of cudaMalloc/cudaFree inside its time loop) cannot let
// the library allocate.  This entry point takes the caller's particle arrays
// and nodal output arrays (device memory the caller owns) and keeps its only
// scratch -- the int64 fixed-point node accumulators -- in one file-scope
// __device__ array below.
//
// Limits and sharing
//   * at most NOALLOC_MAX_NODES control points (64^3 = 262,144); larger grids
//     are rejected with MPM_ERR_BAD_ARG.  The array (16 MiB + 32 bytes) is
//     held by every GPU that loads the library, until the process exits.
//   * every call uses the same array and clears it first; two calls whose
//     kernels overlap on the GPU (different streams, no ordering) race on it
//     and both results are then wrong.
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make
//     that first call before any stream capture.  The address is kept for the
//     life of the process, so the library must not be used across a
//     cudaDeviceReset (which may move the array).
//   * a particle outside the grid, or with a non-finite coordinate, velocity,
//     stress, mass or volume, is skipped (it adds nothing to any node and
//     does not enter the fixed-point bounds) and reported in the caller's
//     device status word: bit 0 outside the grid, bit 1 non-finite.
#include <cstdio>
#include <mutex>

#include "mpm_device.cuh"

namespace mpm {

constexpr int NOALLOC_MAX_NODES = 1 << 18;
constexpr int NA_BOUNDS = 4;   // max m, max vol, max m|v|, max vol*rowsum|sigma| (float bits)

// The only scratch of mpm_gpu_p2g_noalloc: NACC int64 accumulators per node,
// then NA_BOUNDS words for the fixed-point bounds.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[NACC * NOALLOC_MAX_NODES + NA_BOUNDS];

struct NoAllocArgs {
    KGeom<float> g;
    int n;
    const float *x, *v, *s, *m, *vol;   // component blocks of n each: x 3, v 3, s 6
    float *nmass, *nvof, *nmome, *nforce;
    float grav[3];
    float facl;
    float mtol;
    double gshape;
    unsigned long long *scr;
    int *status;   // caller-owned device word: NA_OUTSIDE | NA_NONFINITE
};

constexpr int NA_OUTSIDE = 1;
constexpr int NA_NONFINITE = 2;

// 0 when particle p may be scattered, else the status bit that rejects it.
__device__ __forceinline__ int na_reject(const NoAllocArgs &a, int p) {
    const size_t N = (size_t)a.n;
    float acc = a.m[p] + a.vol[p];
    for (int c = 0; c < 3; c++) acc += a.x[c * N + p] + a.v[c * N + p];
    for (int k = 0; k < 6; k++) acc += a.s[k * N + p];
    if (!isfinite(acc)) return NA_NONFINITE;   // also rejects finite values whose sum overflows
    bool oob = false;
    for (int d = 0; d < 3; d++) (void)cell_of(a.x[d * N + p], a.g, d, oob);
    return oob ? NA_OUTSIDE : 0;
}

__global__ void k_na_clear(unsigned long long *scr, size_t words, int *status) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        scr[i] = 0ull;
    if (blockIdx.x == 0 && threadIdx.x < NA_BOUNDS) scr[NACC * (size_t)NOALLOC_MAX_NODES + threadIdx.x] = 0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0) *status = 0;
}

__device__ __forceinline__ void na_max(unsigned long long *slot, float v) {
    if (!(v >= 0.0f)) v = INFINITY;
    atomicMax(slot, (unsigned long long)__float_as_uint(v));
}

__global__ void k_na_bounds(NoAllocArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    const int rej = na_reject(a, p);
    if (rej) {
        atomicOr(a.status, rej);
        return;
    }
    const size_t N = (size_t)a.n;
    const float m = a.m[p], vol = a.vol[p];
    const float vm = fmaxf(fabsf(a.v[p]), fmaxf(fabsf(a.v[N + p]), fabsf(a.v[2 * N + p])));
    float s[6];
    for (int k = 0; k < 6; k++) s[k] = fabsf(a.s[k * N + p]);
    const float rs = fmaxf(s[0] + s[5] + s[4], fmaxf(s[5] + s[1] + s[3], s[4] + s[3] + s[2]));
    unsigned long long *b = a.scr + NACC * (size_t)NOALLOC_MAX_NODES;
    na_max(b + 0, fabsf(m) * 1.000001f);
    na_max(b + 1, fabsf(vol) * 1.000001f);
    na_max(b + 2, fabsf(m) * vm * 1.000001f);
    na_max(b + 3, fabsf(vol) * rs * 1.000001f);
}

struct NaScales {
    Fix m, v, p, f;
};

__device__ __forceinline__ NaScales na_scales(const NoAllocArgs &a) {
    const unsigned long long *b = a.scr + NACC * (size_t)NOALLOC_MAX_NODES;
    const double nump = (double)a.n;
    const double mmax = (double)__uint_as_float((unsigned)b[0]);
    double gabs = fmax(fabs((double)a.grav[0]), fmax(fabs((double)a.grav[1]), fabs((double)a.grav[2])));
    NaScales s;
    s.m = make_fix(nump * mmax);
    s.v = make_fix(nump * (double)__uint_as_float((unsigned)b[1]));
    s.p = make_fix(nump * (double)__uint_as_float((unsigned)b[2]));
    s.f = make_fix(nump * ((double)__uint_as_float((unsigned)b[3]) * 3.0 * a.gshape + mmax * gabs * fabs((double)a.facl)));
    return s;
}

// Particle2NodeS scatter (module/solid/explicit/var_trans_solid_explicit.cpp:35-70),
// linear shape functions, each contribution added to the scratch in int64.
__global__ void __launch_bounds__(256) k_na_scatter(NoAllocArgs a) {
    __shared__ NaScales S;
    if (threadIdx.x == 0) S = na_scales(a);
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    if (na_reject(a, p)) return;   // reported by k_na_bounds
    const size_t N = (size_t)a.n, NN = (size_t)a.g.nodec;
    const float x0 = a.x[p], x1 = a.x[N + p], x2 = a.x[2 * N + p];
    bool oob = false;
    const int cx = cell_of(x0, a.g, 0, oob), cy = cell_of(x1, a.g, 1, oob), cz = cell_of(x2, a.g, 2, oob);
    Axis<float, 1> ax, ay, az;
    axis_eval<float, 1>(x0, a.g, 0, cx, ax);
    axis_eval<float, 1>(x1, a.g, 1, cy, ay);
    axis_eval<float, 1>(x2, a.g, 2, cz, az);
    const float m = a.m[p], vol = a.vol[p];
    const float v[3] = {a.v[p], a.v[N + p], a.v[2 * N + p]};
    float s[6];
    for (int k = 0; k < 6; k++) s[k] = a.s[k * N + p];
    const float mfx = m * (a.grav[0] * a.facl), mfy = m * (a.grav[1] * a.facl), mfz = m * (a.grav[2] * a.facl);
    for (int k = 0; k < 2; k++)
        for (int j = 0; j < 2; j++)
            for (int i = 0; i < 2; i++) {
                const float wxy = ax.w[i] * ay.w[j];
                const float N_ = wxy * az.w[k];
                const float d0 = ax.dw[i] * ay.w[j] * az.w[k], d1 = ax.w[i] * ay.dw[j] * az.w[k], d2 = wxy * az.dw[k];
                const float Nm = N_ * m;
                const size_t gn = (size_t)(cx + i) + (size_t)a.g.nnc[0] * ((size_t)(cy + j) + (size_t)a.g.nnc[1] * (cz + k));
                long long q[NACC];
                q[0] = fx(Nm, S.m);
                q[1] = fx(N_ * vol, S.v);
                q[2] = fx(Nm * v[0], S.p);
                q[3] = fx(Nm * v[1], S.p);
                q[4] = fx(Nm * v[2], S.p);
                q[5] = fx(-vol * (s[0] * d0 + s[5] * d1 + s[4] * d2) + N_ * mfx, S.f);
                q[6] = fx(-vol * (s[5] * d0 + s[1] * d1 + s[3] * d2) + N_ * mfy, S.f);
                q[7] = fx(-vol * (s[4] * d0 + s[3] * d1 + s[2] * d2) + N_ * mfz, S.f);
                for (int f = 0; f < NACC; f++)
                    if (q[f]) atomicAdd(&a.scr[(size_t)f * NN + gn], (unsigned long long)q[f]);
            }
}

__global__ void k_na_finish(NoAllocArgs a) {
    __shared__ NaScales S;
    if (threadIdx.x == 0) S = na_scales(a);
    __syncthreads();
    const size_t NN = (size_t)a.g.nodec;
    for (size_t n = (size_t)blockIdx.x * blockDim.x + threadIdx.x; n < NN; n += (size_t)gridDim.x * blockDim.x) {
        a.nmass[n] = unfx((long long)a.scr[n], S.m, 0.0f);
        const float vof = unfx((long long)a.scr[NN + n], S.v, 0.0f);
        a.nvof[n] = vof < a.mtol ? 0.0f : vof;   // Particle2NodeS:88
        for (int c = 0; c < 3; c++) {
            a.nmome[c * NN + n] = unfx((long long)a.scr[(2 + c) * NN + n], S.p, 0.0f);
            a.nforce[c * NN + n] = unfx((long long)a.scr[(5 + c) * NN + n], S.f, 0.0f);
        }
    }
}

// Device address of the scratch array, looked up once per device.
static unsigned long long *scratch_address(int dev, cudaError_t *err) {
    static std::mutex mu;
    static unsigned long long *addr[64] = {nullptr};
    std::lock_guard<std::mutex> lock(mu);
    *err = cudaSuccess;
    if (dev < 0 || dev >= 64) {
        *err = cudaErrorInvalidDevice;
        return nullptr;
    }
    if (!addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            *err = e;
            return nullptr;
        }
        addr[dev] = (unsigned long long *)p;
    }
    return addr[dev];
}

}  // namespace mpm

using namespace mpm;

mpm_status mpm_gpu_p2g_noalloc(const mpm_grid_desc *grid, const double *gravity, double facl, double mtol, int64_t n,
                               const float *x, const float *v, const float *stress, const float *mass,
                               const float *vol, float *nmass, float *nvof, float *nmome, float *nforce,
                               int *status, void *stream) {
    if (!grid || !gravity || n < 0 || n > (int64_t)1 << 30) return MPM_ERR_BAD_ARG;
    if (n > 0 && (!x || !v || !stress || !mass || !vol)) return MPM_ERR_BAD_ARG;
    if (!nmass || !nvof || !nmome || !nforce || !status) return MPM_ERR_BAD_ARG;
    NoAllocArgs a;
    long long nodec = 1;
    for (int d = 0; d < 3; d++) {
        if (grid->idimc[d] != 1) return MPM_ERR_UNSUPPORTED;   // linear shape functions only
        if (grid->xyelem[d] <= 0 || !(grid->dxy[d] > 0.0)) return MPM_ERR_BAD_ARG;
        a.g.xmin[d] = (float)grid->xymin[d];
        a.g.dx[d] = (float)grid->dxy[d];
        a.g.inv_dx[d] = (float)(1.0 / grid->dxy[d]);
        a.g.nel[d] = grid->xyelem[d];
        a.g.nnc[d] = grid->xyelem[d] + 1;
        a.g.ntile[d] = 0;
        a.grav[d] = (float)gravity[d];
        nodec *= a.g.nnc[d];
    }
    if (nodec > NOALLOC_MAX_NODES) {
        fprintf(stderr, "mpm_gpu_p2g_noalloc: %lld control points exceed the limit of %d\n", nodec, NOALLOC_MAX_NODES);
        return MPM_ERR_BAD_ARG;
    }
    a.g.nodec = (int)nodec;
    a.n = (int)n;
    a.x = x;
    a.v = v;
    a.s = stress;
    a.m = mass;
    a.vol = vol;
    a.nmass = nmass;
    a.nvof = nvof;
    a.nmome = nmome;
    a.nforce = nforce;
    a.status = status;
    a.facl = (float)facl;
    a.mtol = (float)mtol;
    a.gshape = 0.0;
    for (int d = 0; d < 3; d++) a.gshape = fmax(a.gshape, 1.0 / grid->dxy[d]);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MPM_ERR_CUDA;
    cudaError_t err;
    a.scr = scratch_address(dev, &err);
    if (!a.scr) {
        fprintf(stderr, "mpm_gpu_p2g_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(err));
        return MPM_ERR_CUDA;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const size_t words = (size_t)NACC * (size_t)nodec;
    k_na_clear<<<(int)((words + 255) / 256 < 4096 ? (words + 255) / 256 : 4096), 256, 0, st>>>(a.scr, words, status);
    if (n > 0) {
        const int nb = (int)((n + 255) / 256);
        k_na_bounds<<<nb, 256, 0, st>>>(a);
        k_na_scatter<<<nb, 256, 0, st>>>(a);
    }
    k_na_finish<<<(int)((nodec + 255) / 256 < 4096 ? (nodec + 255) / 256 : 4096), 256, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}
