// Explicit MPM transfer kernels: P2G scatter, grid update, G2P gather with
// the MUSL re-projection, and the position / deformation / stress update.
//
// One explicit step (the sequence of work/src_solid/explicit/main.cpp:39-73):
//   p2g           Particle2NodeS scatter  (module/solid/explicit/var_trans_solid_explicit.cpp:35-70)
//   k_grid1       nvel = p/m + BC, SolveSolid a = f/m + BC, PIC v* = v + dt a,
//                 shifting nei and sum nei^2   (var_trans_solid_explicit.cpp:77-96,
//                 solve_solid_explicit.cpp:8-31, var_trans_solid_explicit.cpp:194-200,
//                 module/material_point.cpp:179-185)
//   g2p_musl      particle velocity gather, MUSL momentum re-scatter, |geup|^2
//                 (var_trans_solid_explicit.cpp:211-240,101-129, material_point.cpp:192-217)
//   k_grid2       MUSL nvel = p/m + BC, shifting b0, clears the accumulators
//                 (var_trans_solid_explicit.cpp:131-146, material_point.cpp:219)
//   k_g2p_update  F update, position update + shift, vol = J vol0, stress
//                 (var_trans_solid_explicit.cpp:247-296,150-185)
//
// Two scatter formulations:
//   * FP32 with linear shape functions (8 nodes per particle): one thread per
//     cell of a 4x4x8-cell brick.  Particles are sorted by (brick, cell, load
//     index), so a thread sums its cell's particles into FP32 registers in a
//     fixed order, writes them to shared memory as cell corners, and a node
//     pass adds the 8 corners of each node in a fixed order before one int64
//     fixed-point RED per node and field.  Runs are bitwise reproducible.
//   * FP64, and quadratic B-splines: particles of a brick chunk convert every
//     contribution to int64 fixed point and scatter into a shared staging box
//     with atomics; the sums are exact and independent of particle order.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "mpm_device.cuh"

namespace mpm {

template <typename R>
struct StepArgs {
    KGeom<R> g;
    Particles<R> P;
    int64_t num;
    const WorkItem *work;
    const int *nwork;
    const int *cstart;          // nbricks * (BRC + 1)
    int *miss;                  // particles that left their sorted cell, processed by a deferred pass
    const int *blist;           // bricks holding particles (brick order) and their count
    const int *nblist;
    const int *tlist;           // active node tiles of this step (tile order) and their count
    const int *ntlist;
    int nbrick[3];
    unsigned long long *acc;    // NACC * nodec
    unsigned long long *acc2;   // 3 * nodec
    unsigned long long *facc;   // nodec (F-bar contexts)
    R *G;                       // gather field for the velocity gather (3 * nodec)
    R *nei;                     // nodec
    R *nvel2;                   // 3 * nodec
    R *nvel_dl, *naccel_dl;     // 3 * nodec each, written only in download mode
    const double *nvol;
    const unsigned char *bcflag;
    const R *bcval;
    unsigned char *tileflag;
    double *eu_part;
    DevCtl *ctl;
    const int *iprop;
    const double *matprop;
    const float *matpropf;      // the same table in FP32 (the FP32 particle kernels)
    R dt, facl, mtol, grav[3];
    int parity;
    int scheme;
    int shifting;
    int all_tiles;              // process every tile in the grid passes (download mode)
    int gnorm;                  // FP32 gathers divide by their weight sum
    int implicit;               // implicit solid: the force fields carry sum N m a (AccelP2G)
    int fbar;                   // F-bar projection: k_grid2 leaves the nodal volume sums to k_fbar_grid
    int sigma_in;               // some material's stress update reads the previous stress (model 0)
    int single_mat;             // one material: every particle's matid is 0
    int fluidj;                 // Tait fluid only: F field 0 holds J - 1, fields 1-8 unused (FP32)
    // traversal directions of the particle kernels: each starts where the
    // previous particle pass ended, so its first bricks are still in L2
    int rev_p2g, rev_g2p, rev_upd;
    double nump;                // particle count as a bound factor
    double mmax;                // max particle mass
    double gshape;              // bound on |dN/dx|
    double gsum;                // bound on sum_i |dN_i/dx|
};

// ----------------------------------------------------------------- helpers
template <typename R>
__device__ __forceinline__ R ld(const R *p) { return __ldg(p); }

__device__ __forceinline__ void tile_coords(int t, const int *nt, int &tx, int &ty, int &tz) {
    tx = t % nt[0];
    ty = (t / nt[0]) % nt[1];
    tz = t / (nt[0] * nt[1]);
}

template <typename R>
__device__ __forceinline__ int tile_of_node(const KGeom<R> &g, int gx, int gy, int gz) {
    return gx / TILE + g.ntile[0] * (gy / TILE + g.ntile[1] * (gz / TILE));
}

template <typename R>
__device__ __forceinline__ size_t node_id(const KGeom<R> &g, int gx, int gy, int gz) {
    return (size_t)gx + (size_t)g.nnc[0] * ((size_t)gy + (size_t)g.nnc[1] * (size_t)gz);
}

// Fixed-point scales.  Computed by one thread of a CTA (FP64 scalar work)
// and shared; producer and consumer kernels derive them from the same
// device-resident bounds, so they agree exactly.

template <typename R>
__device__ void compute_scales(const StepArgs<R> &a, Scales &s) {
    const unsigned *nb = a.ctl->nxt[a.parity];
    double gabs = fmax(fabs((double)a.grav[0]), fmax(fabs((double)a.grav[1]), fabs((double)a.grav[2])));
    s.m = make_fix(a.nump * a.mmax);
    s.v = make_fix(a.nump * (double)bits_f(nb[B_VOLMAX]));
    s.p = make_fix(a.nump * a.mmax * (double)bits_f(nb[B_VMAX]));
    s.f = a.implicit ? make_fix(a.nump * a.mmax * (double)bits_f(nb[B_AMAX]) * 1.0000001)
                     : make_fix(a.nump * ((double)bits_f(nb[B_VOLSMAX]) * 3.0 * a.gshape +
                                          a.mmax * gabs * fabs((double)a.facl)));
    double vb = (double)bits_f(a.ctl->cur[C_GMAX]);
    if (a.scheme == MPM_FLIP) vb = (double)bits_f(nb[B_VMAX]) + fabs((double)a.dt) * vb;
    s.q = make_fix(a.nump * a.mmax * vb * 1.0000001);
    double gb = 2.0 * (double)bits_f(nb[B_VOLMAX]) * a.gsum * (double)bits_f(a.ctl->cur[C_NEIMAX]);
    s.gd = make_fix(a.nump * 3.0 * gb * gb * 1.0000001);
}

// The scales of a step are computed once: the P2G ones by k_step_reset, the
// gather/MUSL ones by the last CTA of k_grid1 (they depend on the grid
// maxima it records).  Kernels copy them into shared memory.
template <typename R>
__device__ __forceinline__ void load_scales_from(const Scales *src, Scales &sh) {
    constexpr int W = (int)(sizeof(Scales) / 4);
    if ((int)threadIdx.x < W) reinterpret_cast<unsigned *>(&sh)[threadIdx.x] = reinterpret_cast<const unsigned *>(src)[threadIdx.x];
    __syncthreads();
}
template <typename R>
__device__ __forceinline__ void load_scales(const StepArgs<R> &a, Scales &sh) {
    load_scales_from<R>(&a.ctl->sc_p2g, sh);
}
template <typename R>
__device__ __forceinline__ void load_scales_musl(const StepArgs<R> &a, Scales &sh) {
    load_scales_from<R>(&a.ctl->sc_musl, sh);
}

// Block-wide reduction (fixed order: deterministic); result valid in thread 0.
template <typename T, typename Op>
__device__ __forceinline__ T block_reduce(T v, Op op, T *sh) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    T r = sh[0];
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) r = op(r, sh[w]);
    return r;
}

struct OpAddD { __device__ double operator()(double a, double b) const { return a + b; } };
struct OpAddL { __device__ long long operator()(long long a, long long b) const { return a + b; } };
struct OpAddI { __device__ int operator()(int a, int b) const { return a + b; } };
struct OpMaxF { __device__ float operator()(float a, float b) const { return fmaxf(a, b); } };

// The eight P2G contributions of one particle to one node
// (StandardVarP2G x3, ComputeInternalForce + ComputeExternalForce,
// material_point.h:223-247, solid_material_point.h:48-73).
template <typename R>
__device__ __forceinline__ void p2g_terms(R N, R d0, R d1, R d2, R m, R vol, const R *v, const R *s, R mfx, R mfy,
                                          R mfz, R *q) {
    const R Nm = N * m;
    q[0] = Nm;
    q[1] = N * vol;
    q[2] = Nm * v[0];
    q[3] = Nm * v[1];
    q[4] = Nm * v[2];
    q[5] = -vol * (s[0] * d0 + s[5] * d1 + s[4] * d2) + N * mfx;
    q[6] = -vol * (s[5] * d0 + s[1] * d1 + s[3] * d2) + N * mfy;
    q[7] = -vol * (s[4] * d0 + s[3] * d1 + s[2] * d2) + N * mfz;
}

template <typename R>
__device__ __forceinline__ void fx_terms(const R *q, const Scales &S, long long *o) {
    o[0] = fx(q[0], S.m);
    o[1] = fx(q[1], S.v);
    o[2] = fx(q[2], S.p);
    o[3] = fx(q[3], S.p);
    o[4] = fx(q[4], S.p);
    o[5] = fx(q[5], S.f);
    o[6] = fx(q[6], S.f);
    o[7] = fx(q[7], S.f);
}

__device__ __forceinline__ void brick_origin(int b, const int *nb, int &ox, int &oy, int &oz) {
    ox = (b % nb[0]) * BRX;
    oy = ((b / nb[0]) % nb[1]) * BRY;
    oz = (b / (nb[0] * nb[1])) * BRZ;
}

// ------------------------------------ tensor-product gather, FP32 linear
// For a field v at the 8 nodes of a cell (v[k][j][i] at node (i, j, k)), the
// value sum_n N_n v_n and the gradient sum_n dN_n/dx v_n evaluated axis by
// axis: the linear weights are (w0, w1) per axis and the node-indexed
// gradients (-1/dx, +1/dx), so the x-gradient at fixed (j, k) is
// (v1 - v0) / dx.  The same sums as node by node with about half the
// operations; outputs a caller does not use are removed by the compiler.
__device__ __forceinline__ void tp_eval(const float (&v)[2][2][2], const Axis<float, 1> &ax,
                                        const Axis<float, 1> &ay, const Axis<float, 1> &az, float &val, float *g) {
    float A[2], Ey[2], Ex[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        float vx[2], dx_[2];
#pragma unroll
        for (int j = 0; j < 2; j++) {
            vx[j] = fmaf(ax.w[1], v[k][j][1], ax.w[0] * v[k][j][0]);
            dx_[j] = v[k][j][1] - v[k][j][0];
        }
        A[k] = fmaf(ay.w[1], vx[1], ay.w[0] * vx[0]);
        Ey[k] = vx[1] - vx[0];
        Ex[k] = fmaf(ay.w[1], dx_[1], ay.w[0] * dx_[0]);
    }
    val = fmaf(az.w[1], A[1], az.w[0] * A[0]);
    g[0] = fmaf(az.w[1], Ex[1], az.w[0] * Ex[0]) * ax.dw[1];
    g[1] = fmaf(az.w[1], Ey[1], az.w[0] * Ey[0]) * ay.dw[1];
    g[2] = (A[1] - A[0]) * az.dw[1];
}

// the cell's 8 node values of field f (nodec values) from one base index
__device__ __forceinline__ void tp_load(const float *f, size_t b0, size_t sy, size_t sz, float (&v)[2][2][2]) {
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int i = 0; i < 2; i++) v[k][j][i] = __ldg(f + b0 + (size_t)i + (j ? sy : 0) + (k ? sz : 0));
}

// ================================================ FP32 linear, per cell
// One CTA per brick, two threads per cell: thread h of cell lc owns the four
// corners of z-layer h (corner c = i + 2 (j + 2 k), k = h), so each thread
// holds 32 FP32 accumulators.  Both threads of a cell read the same
// particles (adjacent lanes, one memory transaction).
constexpr int CELL_SPLIT = 2;
constexpr int CELL_THREADS = BRC * CELL_SPLIT;

// Control-point coordinate xyc[idx][d] along one axis (DefineCpPos,
// module/mesh.h:32-47, on one rank: the open-knot end points of a quadratic
// axis sit on the walls).
template <typename R, int O>
__device__ __forceinline__ R cp_coord(const KGeom<R> &g, int d, int idx) {
    if (O == 1) return g.xmin[d] + g.dx[d] * (R)idx;
    if (idx == 0) return g.xmin[d];
    if (idx == g.nnc[d] - 1) return g.xmin[d] + g.dx[d] * (R)g.nel[d];
    return g.xmin[d] + g.dx[d] * ((R)idx - (R)0.5);
}

// v + A (x_i - x_p): the velocity a TPIC / APIC particle carries to node i
// (TPIC::VarP2G / APIC::VarP2G, module/map_and_interpolate.h:62-77,104-130,
// with the coordinate read as xyc[nid][j]).
template <typename R>
__device__ __forceinline__ void affine_velocity(const R *v, const R *A, R d0, R d1, R d2, R *out) {
#pragma unroll
    for (int c = 0; c < 3; c++) out[c] = v[c] + (A[3 * c] * d0 + A[3 * c + 1] * d1 + A[3 * c + 2] * d2);
}

// One particle of a cell's P2G: FP32 register sums of the four corners of
// z-layer h, or (a particle that left its sorted cell) its own fixed-point
// atomics.  AFF: TPIC / APIC, the momentum carries v + A (x_i - x_p).
template <bool AFF = false>
__device__ __forceinline__ void p2g_particle(const StepArgs<float> &a, const Scales &S, int cx, int cy, int cz, int h,
                                             float x0, float x1, float x2, float m, float vol, const float *v,
                                             const float *s, float fxg, float fyg, float fzg, float (*acc)[4],
                                             int &misses, int &oobs, int defer_p = -1, const float *A = nullptr) {
    bool oob = false;
    const int px = cell_of(x0, a.g, 0, oob), py = cell_of(x1, a.g, 1, oob), pz = cell_of(x2, a.g, 2, oob);
    Axis<float, 1> ax, ay, az;
    axis_eval<float, 1>(x0, a.g, 0, px, ax);
    axis_eval<float, 1>(x1, a.g, 1, py, ay);
    axis_eval<float, 1>(x2, a.g, 2, pz, az);
    const float mfx = m * fxg, mfy = m * fyg, mfz = m * fzg;
    const bool mine = (px == cx) && (py == cy) && (pz == cz);
    // counted once, by the pass that scatters the particle (a deferred one by k_p2g_misses)
    oobs += oob && h == 0 && (mine || defer_p < 0);
    const float wz = h ? az.w[1] : az.w[0], dwz = h ? az.dw[1] : az.dw[0];
    if (!mine) {
        // a particle that left its sorted cell scatters on its own, in the
        // deferred pass (k_p2g_misses) when defer_p names it
        misses += h == 0;
        if (defer_p >= 0) {
            if (h == 0) a.miss[atomicAdd(&a.ctl->n_miss_p2g, 1u)] = defer_p;
            return;
        }
#pragma unroll 1
        for (int c = 0; c < 4; c++) {
            const int i = c & 1, j = c >> 1;
            const float wxy = ax.w[i] * ay.w[j];
            float q[NACC];
            float vn[3] = {v[0], v[1], v[2]};
            if constexpr (AFF)
                affine_velocity(v, A, cp_coord<float, 1>(a.g, 0, px + i) - x0, cp_coord<float, 1>(a.g, 1, py + j) - x1,
                                cp_coord<float, 1>(a.g, 2, pz + h) - x2, vn);
            p2g_terms(wxy * wz, ax.dw[i] * ay.w[j] * wz, ax.w[i] * ay.dw[j] * wz, wxy * dwz, m, vol, vn, s, mfx, mfy,
                      mfz, q);
            long long o[NACC];
            fx_terms(q, S, o);
            const size_t gn = node_id(a.g, px + i, py + j, pz + h);
            for (int f = 0; f < NACC; f++)
                if (o[f]) atomic_add_i64(&a.acc[(size_t)f * a.g.nodec + gn], o[f]);
            a.tileflag[tile_of_node(a.g, px + i, py + j, pz + h)] = 1;
        }
        return;
    }
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const float wxy = ax.w[i] * ay.w[j];
            float q[NACC];
            float vn[3] = {v[0], v[1], v[2]};
            if constexpr (AFF)
                affine_velocity(v, A, cp_coord<float, 1>(a.g, 0, px + i) - x0, cp_coord<float, 1>(a.g, 1, py + j) - x1,
                                cp_coord<float, 1>(a.g, 2, pz + h) - x2, vn);
            p2g_terms(wxy * wz, ax.dw[i] * ay.w[j] * wz, ax.w[i] * ay.dw[j] * wz, wxy * dwz, m, vol, vn, s, mfx, mfy,
                      mfz, q);
            const int c = i + 2 * j;
#pragma unroll
            for (int f = 0; f < NACC; f++) acc[f][c] += q[f];
        }
}

// Node n of a brick's (BRX+1)(BRY+1)(BRZ+1) node box: its grid indices
// (false outside the grid) and, for corner c = i + 2 (j + 2 k), the brick-local
// index of the cell (nx - i, ny - j, nz - k) or -1 where that cell is not in
// the brick.
constexpr int BOX_NODES = (BRX + 1) * (BRY + 1) * (BRZ + 1);
__device__ __forceinline__ bool box_node_cells(const KGeom<float> &g, int n, int ox, int oy, int oz, int &gx,
                                               int &gy, int &gz, int *off) {
    constexpr int NX = BRX + 1, NY = BRY + 1;
    const int nx = n % NX, ny = (n / NX) % NY, nz = n / (NX * NY);
    gx = ox + nx;
    gy = oy + ny;
    gz = oz + nz;
    if (gx >= g.nnc[0] || gy >= g.nnc[1] || gz >= g.nnc[2]) return false;
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int ex = nx - i, ey = ny - j, ez = nz - k;
                off[i + 2 * (j + 2 * k)] = (ex >= 0 && ex < BRX && ey >= 0 && ey < BRY && ez >= 0 && ez < BRZ)
                                               ? ex + BRX * (ey + BRY * ez) : -1;
            }
    return true;
}

// The counters of the cell-P2G kernels: particles that left their sorted cell
// and particles outside the grid.
__device__ __forceinline__ void p2g_counters(const StepArgs<float> &a, int *sh_red, int misses, int oobs) {
    int tot = block_reduce(misses + (oobs << 16), OpAddI(), sh_red);
    if (threadIdx.x == 0 && tot) {
        if (tot & 0xffff) atomicAdd(&a.ctl->tile_misses, (unsigned)(tot & 0xffff));
        if (tot >> 16) atomicAdd(&a.ctl->err_oob, (unsigned)(tot >> 16));
    }
}

// The node pass over the brick's corner sums in shared memory (corner
// f * 8 + c of cell lc in corner[f * 8 + c][lc]): one thread per node of the
// box, all fields; the node's adjacent cells are found once and each field's
// corners are added in the fixed order (k, j, i) = (0, 0, 0) .. (1, 1, 1).
__device__ __forceinline__ void p2g_box_nodes(const StepArgs<float> &a, const Scales &S, const float (*corner)[BRC],
                                              int ox, int oy, int oz) {
    for (int n = threadIdx.x; n < BOX_NODES; n += CELL_THREADS) {
        int gx, gy, gz, off[8];
        if (!box_node_cells(a.g, n, ox, oy, oz, gx, gy, gz, off)) continue;
        // every node of a non-empty brick's box is marked active, so that the
        // grid passes also refresh nodes a particle touches with zero weight
        a.tileflag[tile_of_node(a.g, gx, gy, gz)] = 1;
        const size_t gn = node_id(a.g, gx, gy, gz);
#pragma unroll
        for (int f = 0; f < NACC; f++) {
            float sum = 0.0f;
#pragma unroll
            for (int c = 0; c < 8; c++)
                if (off[c] >= 0) sum += corner[f * 8 + c][off[c]];
            if (sum != 0.0f) {
                const Fix &F = f == 0 ? S.m : f == 1 ? S.v : f <= 4 ? S.p : S.f;
                atomic_add_i64(&a.acc[(size_t)f * a.g.nodec + gn], fx(sum, F));
            }
        }
    }
}

// The end of a cell-P2G brick: this thread's corners of z-layer h to shared
// memory, then the node pass.  COUNT: reduce the counters here (false: the
// caller reduces them once, at the end of a persistent CTA).
template <bool COUNT = true>
__device__ __forceinline__ void p2g_node_pass(const StepArgs<float> &a, const Scales &S, float (*corner)[BRC],
                                              int *sh_red, int lc, int h, int ox, int oy, int oz,
                                              const float (*acc)[4], int misses, int oobs) {
#pragma unroll
    for (int f = 0; f < NACC; f++)
#pragma unroll
        for (int c = 0; c < 4; c++) corner[f * 8 + c + 4 * h][lc] = acc[f][c];
    if (COUNT) p2g_counters(a, sh_red, misses, oobs);
    __syncthreads();
    p2g_box_nodes(a, S, corner, ox, oy, oz);
}

template <int MINB, bool AFF = false>
__global__ void __launch_bounds__(CELL_THREADS, MINB) k_p2g_cell(StepArgs<float> a) {
    __shared__ float corner[NACC * 8][BRC];       // 32 KB
    __shared__ Scales S;
    __shared__ int sh_red[32];
    const int b = blockIdx.x;
    const int lc = threadIdx.x >> 1, h = threadIdx.x & 1;
    const int *cs = a.cstart + (size_t)b * (BRC + 1);
    if (cs[0] == cs[BRC]) return;   // empty brick (uniform across the CTA)
    int ox, oy, oz;
    brick_origin(b, a.nbrick, ox, oy, oz);
    const int cx = ox + (lc % BRX), cy = oy + (lc / BRX) % BRY, cz = oz + lc / (BRX * BRY);
    const int p0 = cs[lc], p1 = cs[lc + 1];
    load_scales(a, S);
    const float fxg = a.grav[0] * a.facl, fyg = a.grav[1] * a.facl, fzg = a.grav[2] * a.facl;
    const Particles<float> &P = a.P;
    float acc[NACC][4];
#pragma unroll
    for (int f = 0; f < NACC; f++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[f][c] = 0.0f;
    int misses = 0, oobs = 0;
    for (int p = p0; p < p1; p++) {
        const float v[3] = {ld(P.v[0] + p), ld(P.v[1] + p), ld(P.v[2] + p)};
        const float s[6] = {ld(P.s[0] + p), ld(P.s[1] + p), ld(P.s[2] + p),
                            ld(P.s[3] + p), ld(P.s[4] + p), ld(P.s[5] + p)};
        float A[AFF ? 9 : 1];
        if constexpr (AFF) {
#pragma unroll
            for (int e = 0; e < 9; e++) A[e] = ld(P.C[e] + p);
        }
        p2g_particle<AFF>(a, S, cx, cy, cz, h, ld(P.x[0] + p), ld(P.x[1] + p), ld(P.x[2] + p), ld(P.m + p),
                          ld(P.vol + p), v, s, fxg, fyg, fzg, acc, misses, oobs, p, A);
    }
    p2g_node_pass(a, S, corner, sh_red, lc, h, ox, oy, oz, acc, misses, oobs);
}

// P2G in moment form.  Within a cell the linear weights are products of
// (1/2 - u) and (1/2 + u) per axis, u in [-1/2, 1/2] the particle's offset
// from the cell centre.  Each thread sums, over its share of the cell's
// particles (the two threads of a cell take alternate particles), the
// moments of q = (m, vol, m v) against {1, u, v, w, uv, uw, vw, uvw} and of
// vol * sigma_ab against the bilinear monomials of the two axes other than
// b: 76 FMAs per particle instead of evaluating eight corner weights and
// gradients.  The pair adds its moments (a + b == b + a, so both threads
// agree), each thread expands them into the four corners of its z-layer,
// and the node pass is the one of k_p2g_cell.  Deterministic: every sum is
// in a fixed order.
// the cell-sum moments q x {1, u, v, w, uv, uw, vw, uvw} of a pair (already
// added across the lanes) expanded into the four corners (i, j, h) of lane h
__device__ __forceinline__ void moments_to_layer(const float *M, int h, float *out) {
    const float sz = h ? 1.0f : -1.0f;
    // the layer's bilinear coefficients over {1, u, v, uv}
    const float L0 = M[0] * 0.125f + sz * M[3] * 0.25f, L1 = M[1] * 0.25f + sz * M[5] * 0.5f,
                L2 = M[2] * 0.25f + sz * M[6] * 0.5f, L3 = M[4] * 0.5f + sz * M[7];
    const float lo = L0 - L2, hi = L0 + L2, dlo = L1 - L3, dhi = L1 + L3;
    out[0] = lo - dlo;   // (i, j) = (0, 0)
    out[1] = lo + dlo;   // (1, 0)
    out[2] = hi - dhi;   // (0, 1)
    out[3] = hi + dhi;   // (1, 1)
}

// The internal force sum_b dN/dx_b (vol sigma_ab) at the four corners
// (i, j, h) of z-layer h, from the stress moments Fm[3 a + b] of vol sigma_ab
// against the bilinear monomials of the two axes other than b: the derivative
// along b carries the sign of b's axis, the bilinear part the other two.
// With the layer's sign sz folded in first, every component is
// K0 + sx K1 + sy K2 + sx sy K3; T[a][i + 2 j].
__device__ __forceinline__ void stress_to_layer(const float (*Fm)[4], int h, const KGeom<float> &g, float (*T)[4]) {
    const float sz = h ? 1.0f : -1.0f;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        const float *Fx = Fm[3 * ax], *Fy = Fm[3 * ax + 1], *Fz = Fm[3 * ax + 2];
        const float ix = g.inv_dx[0], iy = g.inv_dx[1], iz = g.inv_dx[2] * sz;
        // d/dx: sx (Fx0/4 + sz Fx2/2 + sy (Fx1/2 + sz Fx3)); Fx's bilinear axes are (y, z)
        const float ax0 = ix * (Fx[0] * 0.25f + sz * Fx[2] * 0.5f), bx0 = ix * (Fx[1] * 0.5f + sz * Fx[3]);
        // d/dy: sy (Fy0/4 + sz Fy2/2 + sx (Fy1/2 + sz Fy3)); Fy's bilinear axes are (x, z)
        const float ay1 = iy * (Fy[0] * 0.25f + sz * Fy[2] * 0.5f), by1 = iy * (Fy[1] * 0.5f + sz * Fy[3]);
        // d/dz: sz (Fz0/4 + sx Fz1/2 + sy Fz2/2 + sx sy Fz3); Fz's bilinear axes are (x, y)
        const float K0 = iz * Fz[0] * 0.25f, K1 = ax0 + iz * Fz[1] * 0.5f, K2 = ay1 + iz * Fz[2] * 0.5f,
                    K3 = bx0 + by1 + iz * Fz[3];
        const float lo = K0 - K2, hi = K0 + K2, dlo = K1 - K3, dhi = K1 + K3;
        T[ax][0] = lo - dlo;
        T[ax][1] = lo + dlo;
        T[ax][2] = hi - dhi;
        T[ax][3] = hi + dhi;
    }
}

__device__ __forceinline__ float cell_offset_u(float x, const KGeom<float> &g, int d, int c) {
    const float xy = g.xmin[d] + g.dx[d] * (float)c;   // as axis_linear forms x - x_i
    return (x - xy) * g.inv_dx[d] - 0.5f;
}
// the point lies in the cell whose centre the offsets are taken from (false
// for a non-finite offset)
__device__ __forceinline__ bool in_cell(float u, float v, float w) {
    return u >= -0.5f && u < 0.5f && v >= -0.5f && v < 0.5f && w >= -0.5f && w < 0.5f;
}

// the inputs of one particle of the moment-form P2G
struct P2gIn {
    float x[3], m, vol, v[3], s[6];
};
__device__ __forceinline__ void p2g_fetch(const Particles<float> &P, int p, P2gIn &o) {
#pragma unroll
    for (int d = 0; d < 3; d++) o.x[d] = ld(P.x[d] + p);
    o.m = ld(P.m + p);
    o.vol = ld(P.vol + p);
#pragma unroll
    for (int d = 0; d < 3; d++) o.v[d] = ld(P.v[d] + p);
#pragma unroll
    for (int e = 0; e < 6; e++) o.s[e] = ld(P.s[e] + p);
}

template <int MINB, bool LIST, bool PF = false>
__global__ void __launch_bounds__(CELL_THREADS, MINB) k_p2g_cell_mom(StepArgs<float> a) {
    pdl_wait();
    __shared__ float corner[NACC * 8][BRC];       // 32 KB
    __shared__ Scales S;
    __shared__ int sh_red[32];
    load_scales(a, S);
    int misses = 0, oobs = 0;   // over all of this CTA's bricks
    const int nbl = LIST ? *a.nblist : 1;
    for (int li = LIST ? (int)blockIdx.x : 0; li < nbl; li += LIST ? (int)gridDim.x : 1) {
        const int b = LIST ? a.blist[a.rev_p2g ? nbl - 1 - li : li] : (int)blockIdx.x;
        const int lc = threadIdx.x >> 1, h = threadIdx.x & 1;
        const int *cs = a.cstart + (size_t)b * (BRC + 1);
        if (cs[0] == cs[BRC]) continue;   // empty brick (uniform across the CTA)
        int ox, oy, oz;
        brick_origin(b, a.nbrick, ox, oy, oz);
        const int cx = ox + (lc % BRX), cy = oy + (lc / BRX) % BRY, cz = oz + lc / (BRX * BRY);
        const int p0 = cs[lc], p1 = cs[lc + 1];
        const float fxg = a.grav[0] * a.facl, fyg = a.grav[1] * a.facl, fzg = a.grav[2] * a.facl;
        const Particles<float> &P = a.P;
        float M[5][8], Fm[9][4];
#pragma unroll
        for (int f = 0; f < 5; f++)
#pragma unroll
            for (int k = 0; k < 8; k++) M[f][k] = 0.0f;
#pragma unroll
        for (int f = 0; f < 9; f++)
#pragma unroll
            for (int k = 0; k < 4; k++) Fm[f][k] = 0.0f;
        P2gIn nx;
        if (PF && p0 + h < p1) p2g_fetch(P, p0 + h, nx);
        for (int p = p0 + h; p < p1; p += 2) {
            // PF: this particle's inputs were loaded one iteration ahead, and the
            // next one's loads are issued before the work on this one
            P2gIn in;
            if (PF) {
                in = nx;
                if (p + 2 < p1) p2g_fetch(P, p + 2, nx);
            } else {
                p2g_fetch(P, p, in);
            }
            const float x0 = in.x[0], x1 = in.x[1], x2 = in.x[2], m = in.m, vol = in.vol;
            const float *vel = in.v, *sg = in.s;
            // offsets from the sorted cell's centre; a particle outside that
            // cell (or outside the grid, or not finite) scatters in the
            // deferred pass, which also counts the ones outside the grid
            const float u = cell_offset_u(x0, a.g, 0, cx), v = cell_offset_u(x1, a.g, 1, cy),
                        w = cell_offset_u(x2, a.g, 2, cz);
            if (!in_cell(u, v, w)) {
                misses++;
                a.miss[atomicAdd(&a.ctl->n_miss_p2g, 1u)] = p;
                continue;
            }
            const float uv = u * v, uw = u * w, vw = v * w;
            const float mono[8] = {1.0f, u, v, w, uv, uw, vw, uv * w};
            const float q[5] = {m, vol, m * vel[0], m * vel[1], m * vel[2]};
#pragma unroll
            for (int f = 0; f < 5; f++)
#pragma unroll
                for (int k = 0; k < 8; k++) M[f][k] += q[f] * mono[k];
            // vol * sigma_ab, Voigt xx yy zz yz xz xy
            const float vs[9] = {vol * sg[0], vol * sg[5], vol * sg[4], vol * sg[5], vol * sg[1],
                                 vol * sg[3], vol * sg[4], vol * sg[3], vol * sg[2]};
            const float mb[3][4] = {{1.0f, v, w, vw}, {1.0f, u, w, uw}, {1.0f, u, v, uv}};
#pragma unroll
            for (int ab = 0; ab < 9; ab++)
#pragma unroll
                for (int k = 0; k < 4; k++) Fm[ab][k] += vs[ab] * mb[ab % 3][k];
        }
        const unsigned pair = 3u << ((threadIdx.x & 31) & ~1u);
#pragma unroll
        for (int f = 0; f < 5; f++)
#pragma unroll
            for (int k = 0; k < 8; k++) M[f][k] += __shfl_xor_sync(pair, M[f][k], 1);
#pragma unroll
        for (int f = 0; f < 9; f++)
#pragma unroll
            for (int k = 0; k < 4; k++) Fm[f][k] += __shfl_xor_sync(pair, Fm[f][k], 1);
        // corners (i, j, h) of this thread's z-layer
        float acc[NACC][4], T[3][4];
        const float gv[3] = {fxg, fyg, fzg};
#pragma unroll
        for (int f = 0; f < 5; f++) moments_to_layer(M[f], h, acc[f]);
        stress_to_layer(Fm, h, a.g, T);
#pragma unroll
        for (int ax = 0; ax < 3; ax++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[5 + ax][c] = fmaf(acc[0][c], gv[ax], -T[ax][c]);
        p2g_node_pass<false>(a, S, corner, sh_red, lc, h, ox, oy, oz, acc, misses, oobs);
        __syncthreads();   // shared memory is reused by the next brick
    }
    p2g_counters(a, sh_red, misses, oobs);
}

// P2G, one CTA of 128 threads per brick, in two phases per chunk of 128 of
// the brick's particles (a contiguous, coalesced range): (1) thread t takes
// particle t of the chunk and writes its 76 moment terms (see
// k_p2g_cell_mom) to shared memory, or scatters it with atomics if it left
// its sorted cell; (2) thread c adds the terms of its cell's particles in
// particle order into 76 register sums.  Every memory access of the particle
// data is coalesced and the loads of a whole chunk are in flight at once;
// the sums keep a fixed order (deterministic).
constexpr int BCH = 128;                        // particles per chunk
constexpr int NMOM = 76;                        // 40 mass/vol/momentum + 36 stress moments

__global__ void __launch_bounds__(BCH) k_p2g_brick(StepArgs<float> a) {
    __shared__ float T[NMOM][BCH];                 // 38 KB; reused for the corner sums
    __shared__ Scales S;
    __shared__ int sh_red[32];
    __shared__ int scs[BRC + 1];
    const int b = blockIdx.x;
    const int *cs = a.cstart + (size_t)b * (BRC + 1);
    const int P0 = cs[0], P1 = cs[BRC];
    if (P0 == P1) return;
    const int tid = threadIdx.x;
    for (int i = tid; i <= BRC; i += BCH) scs[i] = cs[i];
    int ox, oy, oz;
    brick_origin(b, a.nbrick, ox, oy, oz);
    load_scales(a, S);   // also publishes scs
    const float fxg = a.grav[0] * a.facl, fyg = a.grav[1] * a.facl, fzg = a.grav[2] * a.facl;
    const Particles<float> &P = a.P;
    // this thread's cell (phase 2)
    const int lc = tid;
    const int p0 = scs[lc], p1 = scs[lc + 1];
    float M[NMOM];
#pragma unroll
    for (int k = 0; k < NMOM; k++) M[k] = 0.0f;
    int misses = 0, oobs = 0;
    for (int c0 = P0; c0 < P1; c0 += BCH) {
        // phase 1: one particle per thread
        const int p = c0 + tid;
        if (p < P1) {
            const float x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
            const float m = ld(P.m + p), vol = ld(P.vol + p);
            const float vel[3] = {ld(P.v[0] + p), ld(P.v[1] + p), ld(P.v[2] + p)};
            const float sg[6] = {ld(P.s[0] + p), ld(P.s[1] + p), ld(P.s[2] + p),
                                 ld(P.s[3] + p), ld(P.s[4] + p), ld(P.s[5] + p)};
            bool oob = false;
            const int px = cell_of(x0, a.g, 0, oob), py = cell_of(x1, a.g, 1, oob), pz = cell_of(x2, a.g, 2, oob);
            // mine: the particle sits in the cell whose sorted range holds it
            const int qx = px - ox, qy = py - oy, qz = pz - oz;
            bool mine = (unsigned)qx < (unsigned)BRX && (unsigned)qy < (unsigned)BRY && (unsigned)qz < (unsigned)BRZ;
            if (mine) {
                const int q = qx + BRX * (qy + BRY * qz);
                mine = p >= scs[q] && p < scs[q + 1];
            }
            if (!mine) {
                misses++;
                a.miss[atomicAdd(&a.ctl->n_miss_p2g, 1u)] = p;
#pragma unroll
                for (int k = 0; k < NMOM; k++) T[k][tid] = 0.0f;
            } else {
                oobs += oob;
                const float u = cell_offset_u(x0, a.g, 0, px), v = cell_offset_u(x1, a.g, 1, py),
                            w = cell_offset_u(x2, a.g, 2, pz);
                const float uv = u * v, uw = u * w, vw = v * w;
                const float mono[8] = {1.0f, u, v, w, uv, uw, vw, uv * w};
                const float qv[5] = {m, vol, m * vel[0], m * vel[1], m * vel[2]};
#pragma unroll
                for (int f = 0; f < 5; f++)
#pragma unroll
                    for (int k = 0; k < 8; k++) T[8 * f + k][tid] = qv[f] * mono[k];
                const float vs[9] = {vol * sg[0], vol * sg[5], vol * sg[4], vol * sg[5], vol * sg[1],
                                     vol * sg[3], vol * sg[4], vol * sg[3], vol * sg[2]};
                const float mb[3][4] = {{1.0f, v, w, vw}, {1.0f, u, w, uw}, {1.0f, u, v, uv}};
#pragma unroll
                for (int ab = 0; ab < 9; ab++)
#pragma unroll
                    for (int k = 0; k < 4; k++) T[40 + 4 * ab + k][tid] = vs[ab] * mb[ab % 3][k];
            }
        }
        __syncthreads();
        // phase 2: this thread's cell adds its particles of the chunk in order
        const int q0 = max(p0, c0), q1 = min(p1, c0 + BCH);
        for (int q = q0; q < q1; q++) {
            const int j = q - c0;
#pragma unroll
            for (int k = 0; k < NMOM; k++) M[k] += T[k][j];
        }
        __syncthreads();
    }
    // corners: moments -> the 8 corners of this cell, 8 fields each, into T[f * 8 + corner][cell]
    const float gv[3] = {fxg, fyg, fzg};
#pragma unroll
    for (int kk = 0; kk < 2; kk++)
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int corner = i + 2 * (j + 2 * kk);
                const float sx = i ? 1.0f : -1.0f, sy = j ? 1.0f : -1.0f, sz = kk ? 1.0f : -1.0f;
                float cm[5];
#pragma unroll
                for (int f = 0; f < 5; f++) {
                    const float *Mf = M + 8 * f;
                    cm[f] = Mf[0] * 0.125f + (sx * Mf[1] + sy * Mf[2] + sz * Mf[3]) * 0.25f +
                            (sx * sy * Mf[4] + sx * sz * Mf[5] + sy * sz * Mf[6]) * 0.5f + sx * sy * sz * Mf[7];
                    T[f * 8 + corner][lc] = cm[f];
                }
                const float sb[3] = {sx, sy, sz};
                const float sc[3] = {sy, sx, sx}, sd[3] = {sz, sz, sy};
#pragma unroll
                for (int ax = 0; ax < 3; ax++) {
                    float fi = 0.0f;
#pragma unroll
                    for (int bb = 0; bb < 3; bb++) {
                        const float *F = M + 40 + 4 * (3 * ax + bb);
                        fi += a.g.inv_dx[bb] * sb[bb] *
                              (F[0] * 0.25f + (sc[bb] * F[1] + sd[bb] * F[2]) * 0.5f + sc[bb] * sd[bb] * F[3]);
                    }
                    T[(5 + ax) * 8 + corner][lc] = -fi + cm[0] * gv[ax];
                }
            }
    int tot = block_reduce(misses + (oobs << 16), OpAddI(), sh_red);
    if (threadIdx.x == 0 && tot) {
        if (tot & 0xffff) atomicAdd(&a.ctl->tile_misses, (unsigned)(tot & 0xffff));
        if (tot >> 16) atomicAdd(&a.ctl->err_oob, (unsigned)(tot >> 16));
    }
    __syncthreads();
    constexpr int NX = BRX + 1, NY = BRY + 1, NZ = BRZ + 1, NB = NX * NY * NZ;
    for (int it = threadIdx.x; it < NB * NACC; it += BCH) {
        const int f = it / NB, n = it % NB;
        const int nx = n % NX, ny = (n / NX) % NY, nz = n / (NX * NY);
        const int gx = ox + nx, gy = oy + ny, gz = oz + nz;
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        float sum = 0.0f;
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 2; j++)
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const int ex = nx - i, ey = ny - j, ez = nz - k;
                    if (ex >= 0 && ex < BRX && ey >= 0 && ey < BRY && ez >= 0 && ez < BRZ)
                        sum += T[f * 8 + i + 2 * (j + 2 * k)][ex + BRX * (ey + BRY * ez)];
                }
        if (f == 0) a.tileflag[tile_of_node(a.g, gx, gy, gz)] = 1;
        if (sum != 0.0f) {
            const Fix &F = f == 0 ? S.m : f == 1 ? S.v : f <= 4 ? S.p : S.f;
            atomic_add_i64(&a.acc[(size_t)f * a.g.nodec + node_id(a.g, gx, gy, gz)], fx(sum, F));
        }
    }
}

// The same P2G with the brick's particles brought into shared memory by
// bulk asynchronous copies (TMA, 1-D): the brick's particles are one
// contiguous range (sorted by brick, then cell), copied in chunks of PCH
// particles per field, two chunks in flight.  Each thread then reads its
// cell's particles from shared memory in the same order as k_p2g_cell, so
// both kernels give bitwise the same sums.
constexpr int PCH = 512;                     // particles per staged chunk
constexpr int PNF = 14;                      // x 3, v 3, sigma 6, m, vol
constexpr int PST = PCH + 8;                 // floats per field in a stage (16-byte alignment slack)
constexpr size_t PSTAGE = (size_t)PNF * PST * 4;

template <int MINB>
__global__ void __launch_bounds__(CELL_THREADS, MINB) k_p2g_cell_staged(StepArgs<float> a) {
    extern __shared__ __align__(128) unsigned char dsm[];
    __shared__ float corner[NACC * 8][BRC];       // 32 KB
    __shared__ Scales S;
    __shared__ int sh_red[32];
    __shared__ __align__(8) unsigned long long bar[2];
    const int b = blockIdx.x;
    const int lc = threadIdx.x >> 1, h = threadIdx.x & 1;
    const int *cs = a.cstart + (size_t)b * (BRC + 1);
    const int P0 = cs[0], P1 = cs[BRC];
    if (P0 == P1) return;   // empty brick (uniform across the CTA)
    const Particles<float> &P = a.P;
    const float *src[PNF] = {P.x[0], P.x[1], P.x[2], P.v[0], P.v[1], P.v[2], P.s[0],
                             P.s[1], P.s[2], P.s[3], P.s[4], P.s[5], P.m,    P.vol};
    const int nch = (P1 - P0 + PCH - 1) / PCH;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int k) {
        const int st = k & 1;
        const int c0 = P0 + k * PCH, c1 = min(c0 + PCH, P1);
        const int a0 = c0 & ~3, a1 = (c1 + 3) & ~3;
        const unsigned bytes = (unsigned)(a1 - a0) * 4u;
        float *dst = reinterpret_cast<float *>(dsm + st * PSTAGE);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bar[st], bytes * PNF);
        for (int f = 0; f < PNF; f++) bulk_g2s(dst + f * PST, src[f] + a0, bytes, &bar[st]);
    };
    if (threadIdx.x == 0) issue(0);
    int ox, oy, oz;
    brick_origin(b, a.nbrick, ox, oy, oz);
    const int cx = ox + (lc % BRX), cy = oy + (lc / BRX) % BRY, cz = oz + lc / (BRX * BRY);
    const int p0 = cs[lc], p1 = cs[lc + 1];
    load_scales(a, S);
    const float fxg = a.grav[0] * a.facl, fyg = a.grav[1] * a.facl, fzg = a.grav[2] * a.facl;
    float acc[NACC][4];
#pragma unroll
    for (int f = 0; f < NACC; f++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[f][c] = 0.0f;
    int misses = 0, oobs = 0;
    for (int k = 0; k < nch; k++) {
        const int st = k & 1;
        if (threadIdx.x == 0 && k + 1 < nch) issue(k + 1);
        const bool ok = mbar_wait_bounded(&bar[st], (unsigned)((k >> 1) & 1), 1u << 22);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicAdd(&a.ctl->err_timeout, 1u);
                if (k + 1 < nch) mbar_wait_bounded(&bar[st ^ 1], (unsigned)(((k + 1) >> 1) & 1), 1u << 22);
            }
            __syncthreads();
            return;
        }
        const int c0 = P0 + k * PCH, c1 = min(c0 + PCH, P1);
        const int a0 = c0 & ~3;
        const float *sf = reinterpret_cast<const float *>(dsm + st * PSTAGE);
        const int q0 = max(p0, c0), q1 = min(p1, c1);
        for (int p = q0; p < q1; p++) {
            const int l = p - a0;
            const float v[3] = {sf[3 * PST + l], sf[4 * PST + l], sf[5 * PST + l]};
            const float s[6] = {sf[6 * PST + l], sf[7 * PST + l], sf[8 * PST + l],
                                sf[9 * PST + l], sf[10 * PST + l], sf[11 * PST + l]};
            p2g_particle(a, S, cx, cy, cz, h, sf[l], sf[PST + l], sf[2 * PST + l], sf[12 * PST + l],
                         sf[13 * PST + l], v, s, fxg, fyg, fzg, acc, misses, oobs, p);
        }
        __syncthreads();   // the stage is refilled only after every thread has read it
    }
    p2g_node_pass(a, S, corner, sh_red, lc, h, ox, oy, oz, acc, misses, oobs);
}
// Per-thread gather fields of the cell's four nodes of z-layer h, loaded once.
struct MuslCell {
    float G[3][4], E[4];
};

__device__ __forceinline__ void musl_load_cell(const StepArgs<float> &a, int cx, int cy, int cz, int h, bool any,
                                               MuslCell &C) {
    const size_t N = (size_t)a.g.nodec;
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int c = i + 2 * j;
            if (any) {
                const int gx = min(cx + i, a.g.nnc[0] - 1), gy = min(cy + j, a.g.nnc[1] - 1),
                          gz = min(cz + h, a.g.nnc[2] - 1);
                const size_t gn = node_id(a.g, gx, gy, gz);
#pragma unroll
                for (int d = 0; d < 3; d++) C.G[d][c] = ld(a.G + d * N + gn);
                C.E[c] = ld(a.nei + gn);
            } else {
                C.G[0][c] = C.G[1][c] = C.G[2][c] = C.E[c] = 0.0f;
            }
        }
}

// One particle of the gather + MUSL re-projection: velocity from the four
// nodes of this thread's z-layer plus the partner lane's four, the particle
// velocity write, |geup|^2 and the momentum re-projection sums.
__device__ __forceinline__ void musl_particle(const StepArgs<float> &a, const Scales &S, const MuslCell &C, int cx,
                                              int cy, int cz, int h, int p, float x0, float x1, float x2, float m,
                                              float vol, const float *vold, float (*acc)[4], long long &gacc,
                                              float &vmax) {
    const size_t N = (size_t)a.g.nodec;
    const bool flip = (a.scheme == MPM_FLIP);
    bool oob = false;
    const int px = cell_of(x0, a.g, 0, oob), py = cell_of(x1, a.g, 1, oob), pz = cell_of(x2, a.g, 2, oob);
    Axis<float, 1> ax, ay, az;
    axis_eval<float, 1>(x0, a.g, 0, px, ax);
    axis_eval<float, 1>(x1, a.g, 1, py, ay);
    axis_eval<float, 1>(x2, a.g, 2, pz, az);
    const bool mine = (px == cx) && (py == cy) && (pz == cz);
    if (!mine) {
        // a particle that left its sorted cell: gathered and re-projected by
        // the deferred pass (k_musl_misses); both lanes of the pair skip it
        if (h == 0) a.miss[atomicAdd(&a.ctl->n_miss_musl, 1u)] = p;
        return;
    }
    const float wz = h ? az.w[1] : az.w[0], dwz = h ? az.dw[1] : az.dw[0];
    // partial gathers over this thread's four nodes; the velocity is divided
    // by the sum of the weights, which in FP32 add up to 1 only within a few
    // ulps: that keeps the per-particle bias (the same sign step after step
    // for a particle that stays near its place in the cell) out of it
    float vs[3] = {0.0f, 0.0f, 0.0f}, gu[3] = {0.0f, 0.0f, 0.0f}, ws = 0.0f;
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int c = i + 2 * j;
            const float wxy = ax.w[i] * ay.w[j];
            const float N_ = wxy * wz;
            float gv[3], e;
            if (mine) {
                gv[0] = C.G[0][c];
                gv[1] = C.G[1][c];
                gv[2] = C.G[2][c];
                e = C.E[c];
            } else {
                const size_t gn = node_id(a.g, px + i, py + j, pz + h);
                gv[0] = ld(a.G + gn);
                gv[1] = ld(a.G + N + gn);
                gv[2] = ld(a.G + 2 * N + gn);
                e = ld(a.nei + gn);
            }
            const float wv = flip ? N_ * a.dt : N_;
            ws += wxy;
#pragma unroll
            for (int d = 0; d < 3; d++) vs[d] += wv * gv[d];
            gu[0] += ax.dw[i] * ay.w[j] * wz * e;
            gu[1] += ax.w[i] * ay.dw[j] * wz * e;
            gu[2] += wxy * dwz * e;
        }
    // combine the two halves of the cell (a + b == b + a: both threads agree).
    // Only the cell's own two lanes take part: the other cells of the warp
    // run different particle counts, so a full-warp mask would not converge.
    const unsigned pair = 3u << ((threadIdx.x & 31) & ~1u);
    // sum of the eight weights: the four xy products (the same in both lanes)
    // times each z weight, with no exchange between the lanes
    const float rw = a.gnorm ? rcp_approx(ws * az.w[0] + ws * az.w[1]) : 1.0f;
    float v[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const float other = __shfl_xor_sync(pair, vs[d], 1);
        v[d] = (vs[d] + other) * rw;
        gu[d] += __shfl_xor_sync(pair, gu[d], 1);
    }
    if (flip) {
#pragma unroll
        for (int d = 0; d < 3; d++) v[d] += vold[d];
    }
    if (h == 0) {
        a.P.v[0][p] = v[0];
        a.P.v[1][p] = v[1];
        a.P.v[2][p] = v[2];
        vmax = fmaxf(vmax, fmaxf(fabsf(v[0]), fmaxf(fabsf(v[1]), fabsf(v[2]))));
        const float tv = 2.0f * vol;
        const float g0 = gu[0] * tv, g1 = gu[1] * tv, g2 = gu[2] * tv;
        gacc += fx(g0 * g0 + g1 * g1 + g2 * g2, S.gd);
    }
    // MUSL re-projection of momentum (var_trans_solid_explicit.cpp:108-129)
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int c = i + 2 * j;
            const float Nm = ax.w[i] * ay.w[j] * wz * m;
            if (mine) {
#pragma unroll
                for (int d = 0; d < 3; d++) acc[d][c] += Nm * v[d];
            } else {
                const size_t gn = node_id(a.g, px + i, py + j, pz + h);
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    long long q = fx(Nm * v[d], S.q);
                    if (q) atomic_add_i64(&a.acc2[d * N + gn], q);
                }
            }
        }
}

// the counters of the gather + MUSL kernels: sum |geup|^2 and max |v|
__device__ __forceinline__ void musl_counters(const StepArgs<float> &a, long long *sh_l, float *sh_f, long long gacc,
                                              float vmax) {
    long long gsum = block_reduce(gacc, OpAddL(), sh_l);
    float vm = block_reduce(vmax, OpMaxF(), sh_f);
    if (threadIdx.x == 0) {
        if (gsum) atomicAdd(&a.ctl->geup_acc, (unsigned long long)gsum);
        if (vm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VMAX], vm * 1.000001f);
    }
}

// The re-projection's node pass over the brick's corner sums of m v in
// shared memory (component d, corner c of cell lc in corner[d * 8 + c][lc]),
// in the fixed corner order of p2g_box_nodes.
__device__ __forceinline__ void musl_box_nodes(const StepArgs<float> &a, const Scales &S, const float (*corner)[BRC],
                                               int ox, int oy, int oz) {
    const size_t N = (size_t)a.g.nodec;
    for (int n = threadIdx.x; n < BOX_NODES; n += CELL_THREADS) {
        int gx, gy, gz, off[8];
        if (!box_node_cells(a.g, n, ox, oy, oz, gx, gy, gz, off)) continue;
        const size_t gn = node_id(a.g, gx, gy, gz);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            float sum = 0.0f;
#pragma unroll
            for (int c = 0; c < 8; c++)
                if (off[c] >= 0) sum += corner[d * 8 + c][off[c]];
            if (sum != 0.0f) atomic_add_i64(&a.acc2[d * N + gn], fx(sum, S.q));
        }
    }
}

// The end of a gather + MUSL brick: this thread's corners of z-layer h to
// shared memory, then the node pass.  COUNT as in p2g_node_pass.
template <bool COUNT = true>
__device__ __forceinline__ void musl_node_pass(const StepArgs<float> &a, const Scales &S, float (*corner)[BRC],
                                               long long *sh_l, float *sh_f, int lc, int h, int ox, int oy, int oz,
                                               const float (*acc)[4], long long gacc, float vmax) {
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int c = 0; c < 4; c++) corner[d * 8 + c + 4 * h][lc] = acc[d][c];
    if (COUNT) musl_counters(a, sh_l, sh_f, gacc, vmax);
    __syncthreads();
    musl_box_nodes(a, S, corner, ox, oy, oz);
}

template <int MINB, bool LIST>
__global__ void __launch_bounds__(CELL_THREADS, MINB) k_g2p_musl_cell(StepArgs<float> a) {
    __shared__ float corner[3 * 8][BRC];
    __shared__ Scales S;
    __shared__ long long sh_l[32];
    __shared__ float sh_f[32];
    load_scales_musl(a, S);
    const int nbl = LIST ? *a.nblist : 1;
    for (int li = LIST ? (int)blockIdx.x : 0; li < nbl; li += LIST ? (int)gridDim.x : 1) {
        const int b = LIST ? a.blist[a.rev_g2p ? nbl - 1 - li : li] : (int)blockIdx.x;
        const int lc = threadIdx.x >> 1, h = threadIdx.x & 1;
        const int *cs = a.cstart + (size_t)b * (BRC + 1);
        if (cs[0] == cs[BRC]) continue;   // empty brick (uniform across the CTA)
        int ox, oy, oz;
        brick_origin(b, a.nbrick, ox, oy, oz);
        const int cx = ox + (lc % BRX), cy = oy + (lc / BRX) % BRY, cz = oz + lc / (BRX * BRY);
        const int p0 = cs[lc], p1 = cs[lc + 1];
        const Particles<float> &P = a.P;
        MuslCell C;
        musl_load_cell(a, cx, cy, cz, h, p1 > p0, C);
        float acc[3][4];
#pragma unroll
        for (int d = 0; d < 3; d++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[d][c] = 0.0f;
        long long gacc = 0;
        float vmax = 0.0f;
        const bool flip = (a.scheme == MPM_FLIP);
        for (int p = p0; p < p1; p++) {
            float vold[3] = {0.0f, 0.0f, 0.0f};
            if (flip) {
                vold[0] = ld(P.v[0] + p);
                vold[1] = ld(P.v[1] + p);
                vold[2] = ld(P.v[2] + p);
            }
            musl_particle(a, S, C, cx, cy, cz, h, p, ld(P.x[0] + p), ld(P.x[1] + p), ld(P.x[2] + p), ld(P.m + p),
                          ld(P.vol + p), vold, acc, gacc, vmax);
        }
        musl_node_pass(a, S, corner, sh_l, sh_f, lc, h, ox, oy, oz, acc, gacc, vmax);
        __syncthreads();   // shared memory is reused by the next brick
    }
}

// Gather + MUSL in moment form.  Inside one cell the linear interpolant of a
// nodal field is a trilinear polynomial in the particle's offset (u, v, w)
// from the cell centre (u in [-1/2, 1/2], as in k_p2g_cell_mom).  Each lane of
// a cell's pair forms the eight monomial coefficients over
// {1, u, v, w, uv, uw, vw, uvw} of the gather field (three components) and of
// the shifting field once per cell, by a sum / difference stage per axis
// ((f0 + f1) / 2, f1 - f0); the lanes exchange their z-layer halves for the z
// stage, in the same operand order, so both hold the same coefficients.  A
// constant field gives (f, 0, ..., 0) exactly, so the gathered velocity needs
// no division by the weight sum.  Per particle the gather is 7 FMAs per
// component, the shifting gradient 3 per axis, and the MUSL momentum m v is
// summed against the monomials (24 FMAs) and expanded into corners once per
// cell.  The two lanes take alternate particles.  Deterministic: every sum is
// in a fixed order.  Same sums as the corner form up to FP32 rounding.
__device__ __forceinline__ void lin_stage(float f0, float f1, float &a, float &b) {
    a = (f0 + f1) * 0.5f;
    b = f1 - f0;
}

// f: this lane's z-layer corners f[i + 2 j]; c: coefficients over
// {1, u, v, w, uv, uw, vw, uvw}, the same in both lanes of the pair
__device__ __forceinline__ void trilinear_coeffs(const float *f, int h, unsigned pair, float *c) {
    float a0, b0, a1, b1, L[4];
    lin_stage(f[0], f[1], a0, b0);    // x stage, j = 0
    lin_stage(f[2], f[3], a1, b1);    // x stage, j = 1
    lin_stage(a0, a1, L[0], L[2]);    // y stage: {1, v} of the layer
    lin_stage(b0, b1, L[1], L[3]);    //          {u, uv}
    float lo[4], hi[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float o = __shfl_xor_sync(pair, L[k], 1);
        lo[k] = h ? o : L[k];
        hi[k] = h ? L[k] : o;
    }
    lin_stage(lo[0], hi[0], c[0], c[3]);   // 1, w
    lin_stage(lo[1], hi[1], c[1], c[5]);   // u, uw
    lin_stage(lo[2], hi[2], c[2], c[6]);   // v, vw
    lin_stage(lo[3], hi[3], c[4], c[7]);   // uv, uvw
}

__device__ __forceinline__ float trilinear_eval(const float *c, float u, float v, float w, float uv, float uw,
                                                float vw, float uvw) {
    float r = fmaf(c[1], u, c[0]);
    r = fmaf(c[2], v, r);
    r = fmaf(c[3], w, r);
    r = fmaf(c[4], uv, r);
    r = fmaf(c[5], uw, r);
    r = fmaf(c[6], vw, r);
    return fmaf(c[7], uvw, r);
}

// the inputs of one particle of the moment-form gather (v: FLIP only)
struct MuslIn {
    float x[3], m, vol, v[3];
};
__device__ __forceinline__ void musl_fetch(const Particles<float> &P, int p, bool flip, MuslIn &o) {
    o.x[0] = ld(P.x[0] + p);
    o.x[1] = ld(P.x[1] + p);
    o.x[2] = ld(P.x[2] + p);
    o.m = ld(P.m + p);
    o.vol = ld(P.vol + p);
    o.v[0] = flip ? ld(P.v[0] + p) : 0.0f;
    o.v[1] = flip ? ld(P.v[1] + p) : 0.0f;
    o.v[2] = flip ? ld(P.v[2] + p) : 0.0f;
}

template <int MINB, bool LIST>
__global__ void __launch_bounds__(CELL_THREADS, MINB) k_g2p_musl_mom(StepArgs<float> a) {
    pdl_wait();
    __shared__ float corner[3 * 8][BRC];
    __shared__ Scales S;
    __shared__ long long sh_l[32];
    __shared__ float sh_f[32];
    load_scales_musl(a, S);
    const int nbl = LIST ? *a.nblist : 1;
    const bool flip = (a.scheme == MPM_FLIP);
    const unsigned pair = 3u << ((threadIdx.x & 31) & ~1u);
    long long gacc = 0;   // over all of this CTA's bricks
    float vmax = 0.0f;
    for (int li = LIST ? (int)blockIdx.x : 0; li < nbl; li += LIST ? (int)gridDim.x : 1) {
        const int b = LIST ? a.blist[a.rev_g2p ? nbl - 1 - li : li] : (int)blockIdx.x;
        const int lc = threadIdx.x >> 1, h = threadIdx.x & 1;
        const int *cs = a.cstart + (size_t)b * (BRC + 1);
        if (cs[0] == cs[BRC]) continue;   // empty brick (uniform across the CTA)
        int ox, oy, oz;
        brick_origin(b, a.nbrick, ox, oy, oz);
        const int cx = ox + (lc % BRX), cy = oy + (lc / BRX) % BRY, cz = oz + lc / (BRX * BRY);
        const int p0 = cs[lc], p1 = cs[lc + 1];
        const Particles<float> &P = a.P;
        // the first particle's loads are in flight with the cell's nodal values
        MuslIn nx;
        if (p0 + h < p1) musl_fetch(P, p0 + h, flip, nx);
        float Gc[3][8], Ec[8];
        {
            MuslCell C;
            musl_load_cell(a, cx, cy, cz, h, p1 > p0, C);
#pragma unroll
            for (int d = 0; d < 3; d++) trilinear_coeffs(C.G[d], h, pair, Gc[d]);
            trilinear_coeffs(C.E, h, pair, Ec);
        }
        if (flip) {
            // FLIP gathers the nodal acceleration: v += dt sum N a
#pragma unroll
            for (int d = 0; d < 3; d++)
#pragma unroll
                for (int k = 0; k < 8; k++) Gc[d][k] *= a.dt;
        }
#pragma unroll
        for (int k = 1; k < 8; k++) {
            // the shifting gradient is 2 vol grad(nei); d/dx = inv_dx d/du
            Ec[k] *= 2.0f;
        }
        float M[3][8];
#pragma unroll
        for (int d = 0; d < 3; d++)
#pragma unroll
            for (int k = 0; k < 8; k++) M[d][k] = 0.0f;
        for (int p = p0 + h; p < p1; p += 2) {
            // this particle's inputs, and the next one's loads issued before the work on this one
            const float x0 = nx.x[0], x1 = nx.x[1], x2 = nx.x[2], m = nx.m, vol = nx.vol;
            float vel[3] = {nx.v[0], nx.v[1], nx.v[2]};
            if (p + 2 < p1) musl_fetch(P, p + 2, flip, nx);
            const float u = cell_offset_u(x0, a.g, 0, cx), v = cell_offset_u(x1, a.g, 1, cy),
                        w = cell_offset_u(x2, a.g, 2, cz);
            if (!in_cell(u, v, w)) {
                // a particle outside its sorted cell: the deferred pass (k_musl_misses)
                a.miss[atomicAdd(&a.ctl->n_miss_musl, 1u)] = p;
                continue;
            }
            const float uv = u * v, uw = u * w, vw = v * w, uvw = uv * w;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const float g = trilinear_eval(Gc[d], u, v, w, uv, uw, vw, uvw);
                vel[d] = flip ? vel[d] + g : g;
            }
            P.v[0][p] = vel[0];
            P.v[1][p] = vel[1];
            P.v[2][p] = vel[2];
            vmax = fmaxf(vmax, fmaxf(fabsf(vel[0]), fmaxf(fabsf(vel[1]), fabsf(vel[2]))));
            const float g0 = fmaf(Ec[7], vw, fmaf(Ec[5], w, fmaf(Ec[4], v, Ec[1]))) * a.g.inv_dx[0] * vol;
            const float g1 = fmaf(Ec[7], uw, fmaf(Ec[6], w, fmaf(Ec[4], u, Ec[2]))) * a.g.inv_dx[1] * vol;
            const float g2 = fmaf(Ec[7], uv, fmaf(Ec[6], v, fmaf(Ec[5], u, Ec[3]))) * a.g.inv_dx[2] * vol;
            gacc += fx(g0 * g0 + g1 * g1 + g2 * g2, S.gd);
            const float mono[8] = {1.0f, u, v, w, uv, uw, vw, uvw};
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const float q = m * vel[d];
#pragma unroll
                for (int k = 0; k < 8; k++) M[d][k] = fmaf(q, mono[k], M[d][k]);
            }
        }
        float acc[3][4];
#pragma unroll
        for (int d = 0; d < 3; d++) {
#pragma unroll
            for (int k = 0; k < 8; k++) M[d][k] += __shfl_xor_sync(pair, M[d][k], 1);
            moments_to_layer(M[d], h, acc[d]);
        }
        musl_node_pass<false>(a, S, corner, sh_l, sh_f, lc, h, ox, oy, oz, acc, gacc, vmax);
        __syncthreads();   // shared memory is reused by the next brick
    }
    musl_counters(a, sh_l, sh_f, gacc, vmax);
}

// Gather + MUSL, one CTA of 128 threads per brick, two phases per chunk of
// 128 of the brick's particles as in k_p2g_brick: (1) thread t gathers its
// particle's velocity and shifting gradient from the brick's node box in
// shared memory, writes the velocity (coalesced) and puts the 24 moment
// terms m v x {1, u, v, w, uv, uw, vw, uvw} in shared memory; (2) thread c
// adds its cell's terms in particle order.  Particles that left their
// sorted cell gather from global memory and re-project with atomics.
constexpr int MMOM = 24;

__global__ void __launch_bounds__(BCH) k_musl_brick(StepArgs<float> a) {
    constexpr int NX = BRX + 1, NY = BRY + 1, NZ = BRZ + 1, NBX = NX * NY * NZ;
    __shared__ float T[MMOM][BCH];            // 12 KB; reused for the corner sums
    __shared__ float box[4][NBX];             // G x, y, z and nei of the brick's nodes
    __shared__ Scales S;
    __shared__ long long sh_l[32];
    __shared__ float sh_f[32];
    __shared__ int scs[BRC + 1];
    const int b = blockIdx.x;
    const int *cs = a.cstart + (size_t)b * (BRC + 1);
    const int P0 = cs[0], P1 = cs[BRC];
    if (P0 == P1) return;
    const int tid = threadIdx.x;
    const size_t N = (size_t)a.g.nodec;
    for (int i = tid; i <= BRC; i += BCH) scs[i] = cs[i];
    int ox, oy, oz;
    brick_origin(b, a.nbrick, ox, oy, oz);
    for (int l = tid; l < NBX; l += BCH) {
        const int nx = l % NX, ny = (l / NX) % NY, nz = l / (NX * NY);
        const int gx = min(ox + nx, a.g.nnc[0] - 1), gy = min(oy + ny, a.g.nnc[1] - 1),
                  gz = min(oz + nz, a.g.nnc[2] - 1);
        const size_t gn = node_id(a.g, gx, gy, gz);
        box[0][l] = ld(a.G + gn);
        box[1][l] = ld(a.G + N + gn);
        box[2][l] = ld(a.G + 2 * N + gn);
        box[3][l] = ld(a.nei + gn);
    }
    load_scales_musl(a, S);   // also publishes scs and box
    const Particles<float> &P = a.P;
    const bool flip = (a.scheme == MPM_FLIP);
    const int lc = tid;
    const int p0 = scs[lc], p1 = scs[lc + 1];
    float M[MMOM];
#pragma unroll
    for (int k = 0; k < MMOM; k++) M[k] = 0.0f;
    long long gacc = 0;
    float vmax = 0.0f;
    for (int c0 = P0; c0 < P1; c0 += BCH) {
        const int p = c0 + tid;
        if (p < P1) {
            const float x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
            const float m = ld(P.m + p), vol = ld(P.vol + p);
            bool oob = false;
            const int px = cell_of(x0, a.g, 0, oob), py = cell_of(x1, a.g, 1, oob), pz = cell_of(x2, a.g, 2, oob);
            const int qx = px - ox, qy = py - oy, qz = pz - oz;
            const bool inbox =
                (unsigned)qx < (unsigned)BRX && (unsigned)qy < (unsigned)BRY && (unsigned)qz < (unsigned)BRZ;
            bool mine = inbox;
            if (mine) {
                const int q = qx + BRX * (qy + BRY * qz);
                mine = p >= scs[q] && p < scs[q + 1];
            }
            const float u = cell_offset_u(x0, a.g, 0, px), v = cell_offset_u(x1, a.g, 1, py),
                        w = cell_offset_u(x2, a.g, 2, pz);
            const float wx[2] = {0.5f - u, 0.5f + u}, wy[2] = {0.5f - v, 0.5f + v}, wz[2] = {0.5f - w, 0.5f + w};
            const float dx[2] = {-a.g.inv_dx[0], a.g.inv_dx[0]}, dy[2] = {-a.g.inv_dx[1], a.g.inv_dx[1]},
                        dz[2] = {-a.g.inv_dx[2], a.g.inv_dx[2]};
            float vs[3] = {0.0f, 0.0f, 0.0f}, gu[3] = {0.0f, 0.0f, 0.0f}, ws = 0.0f;
#pragma unroll
            for (int k = 0; k < 2; k++)
#pragma unroll
                for (int j = 0; j < 2; j++)
#pragma unroll
                    for (int i = 0; i < 2; i++) {
                        float gv[3], e;
                        if (inbox) {
                            const int l = (qx + i) + NX * ((qy + j) + NY * (qz + k));
                            gv[0] = box[0][l];
                            gv[1] = box[1][l];
                            gv[2] = box[2][l];
                            e = box[3][l];
                        } else {
                            const size_t gn = node_id(a.g, px + i, py + j, pz + k);
                            gv[0] = ld(a.G + gn);
                            gv[1] = ld(a.G + N + gn);
                            gv[2] = ld(a.G + 2 * N + gn);
                            e = ld(a.nei + gn);
                        }
                        const float wxy = wx[i] * wy[j];
                        const float Nn = wxy * wz[k];
                        const float wv = flip ? Nn * a.dt : Nn;
                        ws += Nn;
#pragma unroll
                        for (int d = 0; d < 3; d++) vs[d] += wv * gv[d];
                        gu[0] += dx[i] * wy[j] * wz[k] * e;
                        gu[1] += wx[i] * dy[j] * wz[k] * e;
                        gu[2] += wxy * dz[k] * e;
                    }
            const float rw = a.gnorm ? rcp_approx(ws) : 1.0f;   // weights summed as gathered (musl_particle)
            float vel[3] = {vs[0] * rw, vs[1] * rw, vs[2] * rw};
            if (flip) {
                vel[0] += ld(P.v[0] + p);
                vel[1] += ld(P.v[1] + p);
                vel[2] += ld(P.v[2] + p);
            }
            P.v[0][p] = vel[0];
            P.v[1][p] = vel[1];
            P.v[2][p] = vel[2];
            vmax = fmaxf(vmax, fmaxf(fabsf(vel[0]), fmaxf(fabsf(vel[1]), fabsf(vel[2]))));
            const float tv = 2.0f * vol;
            const float g0 = gu[0] * tv, g1 = gu[1] * tv, g2 = gu[2] * tv;
            gacc += fx(g0 * g0 + g1 * g1 + g2 * g2, S.gd);
            if (mine) {
                const float uv = u * v;
                const float mono[8] = {1.0f, u, v, w, uv, u * w, v * w, uv * w};
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const float q = m * vel[d];
#pragma unroll
                    for (int k = 0; k < 8; k++) T[8 * d + k][tid] = q * mono[k];
                }
            } else {
#pragma unroll
                for (int k = 0; k < MMOM; k++) T[k][tid] = 0.0f;
#pragma unroll 1
                for (int k = 0; k < 2; k++)
                    for (int j = 0; j < 2; j++)
                        for (int i = 0; i < 2; i++) {
                            const float Nm = wx[i] * wy[j] * wz[k] * m;
                            const size_t gn = node_id(a.g, px + i, py + j, pz + k);
                            for (int d = 0; d < 3; d++) {
                                long long q = fx(Nm * vel[d], S.q);
                                if (q) atomic_add_i64(&a.acc2[d * N + gn], q);
                            }
                        }
            }
        }
        __syncthreads();
        const int q0 = max(p0, c0), q1 = min(p1, c0 + BCH);
        for (int q = q0; q < q1; q++) {
            const int j = q - c0;
#pragma unroll
            for (int k = 0; k < MMOM; k++) M[k] += T[k][j];
        }
        __syncthreads();
    }
    // corners of this cell: T[d * 8 + corner][cell]
#pragma unroll
    for (int kk = 0; kk < 2; kk++)
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int corner = i + 2 * (j + 2 * kk);
                const float sx = i ? 1.0f : -1.0f, sy = j ? 1.0f : -1.0f, sz = kk ? 1.0f : -1.0f;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const float *Md = M + 8 * d;
                    T[d * 8 + corner][lc] = Md[0] * 0.125f + (sx * Md[1] + sy * Md[2] + sz * Md[3]) * 0.25f +
                                            (sx * sy * Md[4] + sx * sz * Md[5] + sy * sz * Md[6]) * 0.5f +
                                            sx * sy * sz * Md[7];
                }
            }
    long long gsum = block_reduce(gacc, OpAddL(), sh_l);
    float vm = block_reduce(vmax, OpMaxF(), sh_f);
    if (threadIdx.x == 0) {
        if (gsum) atomicAdd(&a.ctl->geup_acc, (unsigned long long)gsum);
        if (vm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VMAX], vm * 1.000001f);
    }
    __syncthreads();
    for (int it = threadIdx.x; it < NBX * 3; it += BCH) {
        const int d = it / NBX, n = it % NBX;
        const int nx = n % NX, ny = (n / NX) % NY, nz = n / (NX * NY);
        const int gx = ox + nx, gy = oy + ny, gz = oz + nz;
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        float sum = 0.0f;
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 2; j++)
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const int ex = nx - i, ey = ny - j, ez = nz - k;
                    if (ex >= 0 && ex < BRX && ey >= 0 && ey < BRY && ez >= 0 && ez < BRZ)
                        sum += T[d * 8 + i + 2 * (j + 2 * k)][ex + BRX * (ey + BRY * ez)];
                }
        if (sum != 0.0f) atomic_add_i64(&a.acc2[d * N + node_id(a.g, gx, gy, gz)], fx(sum, S.q));
    }
}

// The gather + MUSL with the brick's x, m, vol and (FLIP) v staged in shared
// memory by bulk asynchronous copies, as k_p2g_cell_staged; same order of
// operations as k_g2p_musl_cell, so the same results bit for bit.
constexpr int MNF = 8;                       // x 3, m, vol, v 3
constexpr size_t MSTAGE = (size_t)MNF * PST * 4;

template <int MINB>
__global__ void __launch_bounds__(CELL_THREADS, MINB) k_g2p_musl_cell_staged(StepArgs<float> a) {
    extern __shared__ __align__(128) unsigned char dsm[];
    __shared__ float corner[3 * 8][BRC];
    __shared__ Scales S;
    __shared__ long long sh_l[32];
    __shared__ float sh_f[32];
    __shared__ __align__(8) unsigned long long bar[2];
    const int b = blockIdx.x;
    const int lc = threadIdx.x >> 1, h = threadIdx.x & 1;
    const int *cs = a.cstart + (size_t)b * (BRC + 1);
    const int P0 = cs[0], P1 = cs[BRC];
    if (P0 == P1) return;
    const Particles<float> &P = a.P;
    const bool flip = (a.scheme == MPM_FLIP);
    const int nf = flip ? MNF : 5;
    const float *src[MNF] = {P.x[0], P.x[1], P.x[2], P.m, P.vol, P.v[0], P.v[1], P.v[2]};
    const int nch = (P1 - P0 + PCH - 1) / PCH;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int k) {
        const int st = k & 1;
        const int c0 = P0 + k * PCH, c1 = min(c0 + PCH, P1);
        const int a0 = c0 & ~3, a1 = (c1 + 3) & ~3;
        const unsigned bytes = (unsigned)(a1 - a0) * 4u;
        float *dst = reinterpret_cast<float *>(dsm + st * MSTAGE);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bar[st], bytes * nf);
        for (int f = 0; f < nf; f++) bulk_g2s(dst + f * PST, src[f] + a0, bytes, &bar[st]);
    };
    if (threadIdx.x == 0) issue(0);
    int ox, oy, oz;
    brick_origin(b, a.nbrick, ox, oy, oz);
    const int cx = ox + (lc % BRX), cy = oy + (lc / BRX) % BRY, cz = oz + lc / (BRX * BRY);
    const int p0 = cs[lc], p1 = cs[lc + 1];
    load_scales_musl(a, S);
    MuslCell C;
    musl_load_cell(a, cx, cy, cz, h, p1 > p0, C);
    float acc[3][4];
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[d][c] = 0.0f;
    long long gacc = 0;
    float vmax = 0.0f;
    for (int k = 0; k < nch; k++) {
        const int st = k & 1;
        if (threadIdx.x == 0 && k + 1 < nch) issue(k + 1);
        const bool ok = mbar_wait_bounded(&bar[st], (unsigned)((k >> 1) & 1), 1u << 22);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                atomicAdd(&a.ctl->err_timeout, 1u);
                if (k + 1 < nch) mbar_wait_bounded(&bar[st ^ 1], (unsigned)(((k + 1) >> 1) & 1), 1u << 22);
            }
            __syncthreads();
            return;
        }
        const int c0 = P0 + k * PCH, c1 = min(c0 + PCH, P1);
        const int a0 = c0 & ~3;
        const float *sf = reinterpret_cast<const float *>(dsm + st * MSTAGE);
        const int q0 = max(p0, c0), q1 = min(p1, c1);
        for (int p = q0; p < q1; p++) {
            const int l = p - a0;
            float vold[3] = {0.0f, 0.0f, 0.0f};
            if (flip) {
                vold[0] = sf[5 * PST + l];
                vold[1] = sf[6 * PST + l];
                vold[2] = sf[7 * PST + l];
            }
            musl_particle(a, S, C, cx, cy, cz, h, p, sf[l], sf[PST + l], sf[2 * PST + l], sf[3 * PST + l],
                          sf[4 * PST + l], vold, acc, gacc, vmax);
        }
        __syncthreads();
    }
    musl_node_pass(a, S, corner, sh_l, sh_f, lc, h, ox, oy, oz, acc, gacc, vmax);
}

// Deferred passes for the particles that left their sorted cell since the
// last re-sort: fixed-point atomics (order independent, so the results do
// not depend on the queue order); the P2G with eight threads per queued
// particle, the gather + MUSL with one.
template <bool AFF = false>
__global__ void __launch_bounds__(256) k_p2g_misses(StepArgs<float> a) {
    pdl_wait();
    __shared__ Scales S;
    __shared__ int sh_red[32];
    load_scales(a, S);
    const unsigned n = a.ctl->n_miss_p2g;
    const float fxg = a.grav[0] * a.facl, fyg = a.grav[1] * a.facl, fzg = a.grav[2] * a.facl;
    const Particles<float> &P = a.P;
    int oobs = 0;
    // eight threads per deferred particle, one per corner (i, j, h): the
    // corner's terms are those of p2g_particle's scatter path, and the int64
    // sums make the result independent of which thread adds them
    for (size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x; g < 8 * (size_t)n;
         g += (size_t)gridDim.x * blockDim.x) {
        const int p = a.miss[g >> 3];
        const int ci = g & 1, cj = (g >> 1) & 1, h = (g >> 2) & 1;
        const float x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p), m = ld(P.m + p),
                    vol = ld(P.vol + p);
        const float vel[3] = {ld(P.v[0] + p), ld(P.v[1] + p), ld(P.v[2] + p)};
        const float sg[6] = {ld(P.s[0] + p), ld(P.s[1] + p), ld(P.s[2] + p),
                             ld(P.s[3] + p), ld(P.s[4] + p), ld(P.s[5] + p)};
        bool oob = false;
        const int px = cell_of(x0, a.g, 0, oob), py = cell_of(x1, a.g, 1, oob), pz = cell_of(x2, a.g, 2, oob);
        oobs += oob && (g & 7) == 0;
        Axis<float, 1> ax, ay, az;
        axis_eval<float, 1>(x0, a.g, 0, px, ax);
        axis_eval<float, 1>(x1, a.g, 1, py, ay);
        axis_eval<float, 1>(x2, a.g, 2, pz, az);
        const float mfx = m * fxg, mfy = m * fyg, mfz = m * fzg;
        const float wz = h ? az.w[1] : az.w[0], dwz = h ? az.dw[1] : az.dw[0];
        const float wxy = ax.w[ci] * ay.w[cj];
        float vn[3] = {vel[0], vel[1], vel[2]};
        if constexpr (AFF) {
            float A[9];
#pragma unroll
            for (int e = 0; e < 9; e++) A[e] = ld(P.C[e] + p);
            affine_velocity(vel, A, cp_coord<float, 1>(a.g, 0, px + ci) - x0, cp_coord<float, 1>(a.g, 1, py + cj) - x1,
                            cp_coord<float, 1>(a.g, 2, pz + h) - x2, vn);
        }
        float q[NACC];
        p2g_terms(wxy * wz, ax.dw[ci] * ay.w[cj] * wz, ax.w[ci] * ay.dw[cj] * wz, wxy * dwz, m, vol, vn, sg, mfx, mfy,
                  mfz, q);
        long long o[NACC];
        fx_terms(q, S, o);
        const size_t gn = node_id(a.g, px + ci, py + cj, pz + h);
#pragma unroll
        for (int f = 0; f < NACC; f++)
            if (o[f]) atomic_add_i64(&a.acc[(size_t)f * a.g.nodec + gn], o[f]);
        a.tileflag[tile_of_node(a.g, px + ci, py + cj, pz + h)] = 1;
    }
    // the particles outside the grid (every one of them is deferred by the
    // moment-form P2G)
    const int tot = block_reduce(oobs, OpAddI(), sh_red);
    if (threadIdx.x == 0 && tot) atomicAdd(&a.ctl->err_oob, (unsigned)tot);
}

__global__ void __launch_bounds__(256) k_musl_misses(StepArgs<float> a) {
    pdl_wait();
    __shared__ Scales S;
    __shared__ long long sh_l[32];
    __shared__ float sh_f[32];
    load_scales_musl(a, S);
    const unsigned n = a.ctl->n_miss_musl;
    const size_t N = (size_t)a.g.nodec;
    const bool flip = (a.scheme == MPM_FLIP);
    const Particles<float> &P = a.P;
    long long gacc = 0;
    float vmax = 0.0f;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = a.miss[i];
        const float x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        const float m = ld(P.m + p), vol = ld(P.vol + p);
        bool oob = false;
        const int px = cell_of(x0, a.g, 0, oob), py = cell_of(x1, a.g, 1, oob), pz = cell_of(x2, a.g, 2, oob);
        Axis<float, 1> ax, ay, az;
        axis_eval<float, 1>(x0, a.g, 0, px, ax);
        axis_eval<float, 1>(x1, a.g, 1, py, ay);
        axis_eval<float, 1>(x2, a.g, 2, pz, az);
        float v[3] = {0.0f, 0.0f, 0.0f}, gu[3] = {0.0f, 0.0f, 0.0f}, ws = 0.0f;
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++)
                for (int ii = 0; ii < 2; ii++) {
                    const size_t gn = node_id(a.g, px + ii, py + j, pz + k);
                    const float wxy = ax.w[ii] * ay.w[j];
                    const float N_ = wxy * az.w[k];
                    const float wv = flip ? N_ * a.dt : N_;
                    const float e = ld(a.nei + gn);
                    ws += N_;
#pragma unroll
                    for (int d = 0; d < 3; d++) v[d] += wv * ld(a.G + d * N + gn);
                    gu[0] += ax.dw[ii] * ay.w[j] * az.w[k] * e;
                    gu[1] += ax.w[ii] * ay.dw[j] * az.w[k] * e;
                    gu[2] += wxy * az.dw[k] * e;
                }
        const float rw = a.gnorm ? rcp_approx(ws) : 1.0f;   // divided by the weights it used, as musl_particle
#pragma unroll
        for (int d = 0; d < 3; d++) v[d] *= rw;
        if (flip) {
#pragma unroll
            for (int d = 0; d < 3; d++) v[d] += ld(P.v[d] + p);
        }
        P.v[0][p] = v[0];
        P.v[1][p] = v[1];
        P.v[2][p] = v[2];
        vmax = fmaxf(vmax, fmaxf(fabsf(v[0]), fmaxf(fabsf(v[1]), fabsf(v[2]))));
        const float tv = 2.0f * vol;
        const float g0 = gu[0] * tv, g1 = gu[1] * tv, g2 = gu[2] * tv;
        gacc += fx(g0 * g0 + g1 * g1 + g2 * g2, S.gd);
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++)
                for (int ii = 0; ii < 2; ii++) {
                    const float Nm = ax.w[ii] * ay.w[j] * az.w[k] * m;
                    const size_t gn = node_id(a.g, px + ii, py + j, pz + k);
                    for (int d = 0; d < 3; d++) {
                        const long long q = fx(Nm * v[d], S.q);
                        if (q) atomic_add_i64(&a.acc2[d * N + gn], q);
                    }
                }
    }
    const long long gsum = block_reduce(gacc, OpAddL(), sh_l);
    const float vm = block_reduce(vmax, OpMaxF(), sh_f);
    if (threadIdx.x == 0) {
        if (gsum) atomicAdd(&a.ctl->geup_acc, (unsigned long long)gsum);
        if (vm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VMAX], vm * 1.000001f);
    }
}

// Launched before the P2G of every step: records the P2G scales (for result
// downloads) and resets the per-step device counters.
template <typename R>
__global__ void k_step_reset(StepArgs<R> a) {
    pdl_wait();
    Scales s;
    compute_scales(a, s);
    DevCtl *ctl = a.ctl;
    ctl->p2g_inv[0] = s.m.inv;
    ctl->p2g_inv[1] = s.v.inv;
    ctl->p2g_inv[2] = s.p.inv;
    ctl->p2g_inv[3] = s.f.inv;
    ctl->sc_p2g = s;
    ctl->n_miss_p2g = 0u;
    ctl->n_miss_musl = 0u;
    for (int k = 0; k < B_NB; k++) ctl->nxt[a.parity ^ 1][k] = 0u;
    for (int k = 0; k < C_NC; k++) ctl->cur[k] = 0u;
    ctl->geup_acc = 0ull;
}

// ================================================= any order, staging box
// One CTA per work item (a chunk of one brick's particles); every
// contribution is converted to int64 and added into a shared box of the
// brick's nodes (exact, order independent).
template <typename R, int OX, int OY, int OZ, bool AFF = false>
__global__ void __launch_bounds__(256) k_p2g_box(StepArgs<R> a) {
    constexpr int BX = BRX + OX, BY = BRY + OY, BZ = BRZ + OZ, BOX = BX * BY * BZ;
    extern __shared__ unsigned long long sacc[];   // NACC * BOX
    __shared__ Scales S;
    __shared__ int sh_red[32];
    if ((int)blockIdx.x >= *a.nwork) return;
    const WorkItem w = a.work[blockIdx.x];
    int ox, oy, oz;
    brick_origin(w.tile, a.nbrick, ox, oy, oz);
    for (int i = threadIdx.x; i < NACC * BOX; i += blockDim.x) sacc[i] = 0ull;
    load_scales(a, S);
    const R fxg = a.grav[0] * a.facl, fyg = a.grav[1] * a.facl, fzg = a.grav[2] * a.facl;
    const Particles<R> &P = a.P;
    int misses = 0, oobs = 0;
    for (int p = w.begin + threadIdx.x; p < w.end; p += blockDim.x) {
        const R x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        const int cx = cell_of(x0, a.g, 0, oob), cy = cell_of(x1, a.g, 1, oob), cz = cell_of(x2, a.g, 2, oob);
        oobs += oob;
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        axis_eval<R, OX>(x0, a.g, 0, cx, ax);
        axis_eval<R, OY>(x1, a.g, 1, cy, ay);
        axis_eval<R, OZ>(x2, a.g, 2, cz, az);
        const R m = ld(P.m + p), vol = ld(P.vol + p);
        const R v[3] = {ld(P.v[0] + p), ld(P.v[1] + p), ld(P.v[2] + p)};
        const R s[6] = {ld(P.s[0] + p), ld(P.s[1] + p), ld(P.s[2] + p),
                        ld(P.s[3] + p), ld(P.s[4] + p), ld(P.s[5] + p)};
        const R mfx = m * fxg, mfy = m * fyg, mfz = m * fzg;
        const int lx = cx - ox, ly = cy - oy, lz = cz - oz;
        const bool in = (unsigned)lx < (unsigned)BRX && (unsigned)ly < (unsigned)BRY && (unsigned)lz < (unsigned)BRZ;
        misses += !in;
        R pa[3] = {(R)0, (R)0, (R)0};
        if (a.implicit) {
            pa[0] = ld(P.a[0] + p); pa[1] = ld(P.a[1] + p); pa[2] = ld(P.a[2] + p);
        }
        R A[AFF ? 9 : 1];
        if constexpr (AFF) {
#pragma unroll
            for (int e = 0; e < 9; e++) A[e] = ld(P.C[e] + p);
        }
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R wxy = ax.w[i] * ay.w[j];
                    R q[NACC];
                    R vn[3] = {v[0], v[1], v[2]};
                    if constexpr (AFF)
                        affine_velocity(v, A, cp_coord<R, OX>(a.g, 0, cx + i) - x0, cp_coord<R, OY>(a.g, 1, cy + j) - x1,
                                        cp_coord<R, OZ>(a.g, 2, cz + k) - x2, vn);
                    p2g_terms(wxy * az.w[k], ax.dw[i] * ay.w[j] * az.w[k], ax.w[i] * ay.dw[j] * az.w[k],
                              wxy * az.dw[k], m, vol, vn, s, mfx, mfy, mfz, q);
                    if (a.implicit) {
                        // AccelP2G (map_and_interpolate.cpp:42-53): nforce += N m a
                        const R Nm = wxy * az.w[k] * m;
                        q[5] = Nm * pa[0];
                        q[6] = Nm * pa[1];
                        q[7] = Nm * pa[2];
                    }
                    long long o[NACC];
                    fx_terms(q, S, o);
                    if (in) {
                        const int li = (lx + i) + BX * ((ly + j) + BY * (lz + k));
#pragma unroll
                        for (int f = 0; f < NACC; f++) atomic_add_i64(&sacc[f * BOX + li], o[f]);
                    } else {
                        const size_t gn = node_id(a.g, cx + i, cy + j, cz + k);
#pragma unroll
                        for (int f = 0; f < NACC; f++) atomic_add_i64(&a.acc[(size_t)f * a.g.nodec + gn], o[f]);
                        a.tileflag[tile_of_node(a.g, cx + i, cy + j, cz + k)] = 1;
                    }
                }
    }
    int tot = block_reduce(misses + (oobs << 16), OpAddI(), sh_red);
    if (threadIdx.x == 0 && tot) {
        if (tot & 0xffff) atomicAdd(&a.ctl->tile_misses, (unsigned)(tot & 0xffff));
        if (tot >> 16) atomicAdd(&a.ctl->err_oob, (unsigned)(tot >> 16));
    }
    __syncthreads();
    for (int li = threadIdx.x; li < BOX; li += blockDim.x) {
        const int lx = li % BX, ly = (li / BX) % BY, lz = li / (BX * BY);
        const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        const size_t gn = node_id(a.g, gx, gy, gz);
#pragma unroll
        for (int f = 0; f < NACC; f++) {
            unsigned long long v = sacc[f * BOX + li];
            if (v) atomicAdd(&a.acc[(size_t)f * a.g.nodec + gn], v);
        }
        a.tileflag[tile_of_node(a.g, gx, gy, gz)] = 1;
    }
}

template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(256) k_g2p_musl_box(StepArgs<R> a) {
    constexpr int BX = BRX + OX, BY = BRY + OY, BZ = BRZ + OZ, BOX = BX * BY * BZ;
    extern __shared__ unsigned long long sacc[];   // 3 * BOX
    __shared__ Scales S;
    __shared__ long long sh_l[32];
    __shared__ float sh_f[32];
    if ((int)blockIdx.x >= *a.nwork) return;
    const WorkItem w = a.work[blockIdx.x];
    int ox, oy, oz;
    brick_origin(w.tile, a.nbrick, ox, oy, oz);
    for (int i = threadIdx.x; i < 3 * BOX; i += blockDim.x) sacc[i] = 0ull;
    load_scales_musl(a, S);
    const size_t N = (size_t)a.g.nodec;
    const Particles<R> &P = a.P;
    const bool flip = (a.scheme == MPM_FLIP);
    long long gacc = 0;
    float vmax = 0.0f;
    for (int p = w.begin + threadIdx.x; p < w.end; p += blockDim.x) {
        const R x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        const int cx = cell_of(x0, a.g, 0, oob), cy = cell_of(x1, a.g, 1, oob), cz = cell_of(x2, a.g, 2, oob);
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        axis_eval<R, OX>(x0, a.g, 0, cx, ax);
        axis_eval<R, OY>(x1, a.g, 1, cy, ay);
        axis_eval<R, OZ>(x2, a.g, 2, cz, az);
        const R m = ld(P.m + p), vol = ld(P.vol + p);
        R v[3];
        if (flip) {
            v[0] = ld(P.v[0] + p); v[1] = ld(P.v[1] + p); v[2] = ld(P.v[2] + p);
        } else {
            v[0] = v[1] = v[2] = (R)0;
        }
        R gu[3] = {(R)0, (R)0, (R)0};
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R wxy = ax.w[i] * ay.w[j];
                    const R N_ = wxy * az.w[k];
                    const size_t gn = node_id(a.g, cx + i, cy + j, cz + k);
                    if (flip) {
                        const R Nd = N_ * a.dt;
#pragma unroll
                        for (int d = 0; d < 3; d++) v[d] += Nd * ld(a.G + d * N + gn);
                    } else {
#pragma unroll
                        for (int d = 0; d < 3; d++) v[d] += N_ * ld(a.G + d * N + gn);
                    }
                    const R e = ld(a.nei + gn);
                    gu[0] += ax.dw[i] * ay.w[j] * az.w[k] * e;
                    gu[1] += ax.w[i] * ay.dw[j] * az.w[k] * e;
                    gu[2] += wxy * az.dw[k] * e;
                }
        P.v[0][p] = v[0];
        P.v[1][p] = v[1];
        P.v[2][p] = v[2];
        vmax = fmaxf(vmax, fmaxf(fabsf((float)v[0]), fmaxf(fabsf((float)v[1]), fabsf((float)v[2]))));
        const R tv = (R)2 * vol;
        const R g0 = gu[0] * tv, g1 = gu[1] * tv, g2 = gu[2] * tv;
        gacc += fx(g0 * g0 + g1 * g1 + g2 * g2, S.gd);
        const int lx = cx - ox, ly = cy - oy, lz = cz - oz;
        const bool in = (unsigned)lx < (unsigned)BRX && (unsigned)ly < (unsigned)BRY && (unsigned)lz < (unsigned)BRZ;
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R Nm = ax.w[i] * ay.w[j] * az.w[k] * m;
                    const long long q0 = fx(Nm * v[0], S.q), q1 = fx(Nm * v[1], S.q), q2 = fx(Nm * v[2], S.q);
                    if (in) {
                        const int li = (lx + i) + BX * ((ly + j) + BY * (lz + k));
                        atomic_add_i64(&sacc[li], q0);
                        atomic_add_i64(&sacc[BOX + li], q1);
                        atomic_add_i64(&sacc[2 * BOX + li], q2);
                    } else {
                        const size_t gn = node_id(a.g, cx + i, cy + j, cz + k);
                        atomic_add_i64(&a.acc2[gn], q0);
                        atomic_add_i64(&a.acc2[N + gn], q1);
                        atomic_add_i64(&a.acc2[2 * N + gn], q2);
                    }
                }
    }
    long long gsum = block_reduce(gacc, OpAddL(), sh_l);
    float vm = block_reduce(vmax, OpMaxF(), sh_f);
    if (threadIdx.x == 0) {
        if (gsum) atomicAdd(&a.ctl->geup_acc, (unsigned long long)gsum);
        if (vm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VMAX], vm * 1.000001f);
    }
    __syncthreads();
    for (int li = threadIdx.x; li < BOX; li += blockDim.x) {
        const int lx = li % BX, ly = (li / BX) % BY, lz = li / (BX * BY);
        const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        const size_t gn = node_id(a.g, gx, gy, gz);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            unsigned long long v = sacc[d * BOX + li];
            if (v) atomicAdd(&a.acc2[d * N + gn], v);
        }
    }
}

// ================================================= TPIC / APIC gather + MUSL
// Three launches replace the gather + MUSL kernel for the affine schemes:
// the gather of the velocity (PIC) and of the affine matrix, one thread per
// particle; a one-thread kernel that sets the MUSL fixed-point scale from the
// bound the gather recorded (APIC's D^-1 has no a-priori bound); the MUSL
// scatter of m (v + A (x_i - x_p)) through the brick staging box.
//   TPIC (TPIC::VarGradG2P, map_and_interpolate.h:79-98): A[c][j] = sum_i dN_i/dx_j G_i,c
//   APIC (APIC::VarBmatG2P / DmatG2P / InvDmatG2P, map_and_interpolate.h:132-172):
//     B[c][j] = sum_i N_i G_i,c d_i,j, D[a][b] = sum_i N_i d_i,a d_i,b, A = B D^-1
// with G the PIC gather field (nvel + dt naccel) and d_i = xyc_i - x_p.  The
// recorded bound max_p,c (|v_c| + sum_j |A_cj| dmax_j), dmax_j the largest
// node-particle distance along axis j (dx linear, 1.5 dx quadratic), covers
// every momentum contribution of this MUSL and of the next step's P2G.
// APIC weights and node offsets along one axis.  Linear axes take each
// weight from its own node distance (w_i = r_{i+1} / dx, w_{i+1} = r_i / dx
// with r_i = x - x_i, r_{i+1} = x_{i+1} - x): equal to 1 - |x - x_node| / dx
// in exact arithmetic, but a particle close to a grid plane keeps its small
// weight to full relative precision, so B and D (whose terms cancel to
// O(r dx) there) stay accurate; quadratic axes, whose D is well conditioned,
// use the B-spline weights.  On a linear axis both distances are kept at
// least 1e-7 dx (FP32) / 1e-12 dx (FP64): a particle exactly on a grid plane
// (common in FP32) would make D singular, and there B D^-1 has a finite
// limit (for multilinear shape functions it equals the velocity gradient at
// any position inside the cell), which the floored distances give.
template <typename R, int O>
__device__ __forceinline__ void apic_axis(const KGeom<R> &g, int d, int c, R x, const Axis<R, O> &ax, R *w, R *dd) {
    if (O == 1) {
        const R tiny = (sizeof(R) == 4 ? (R)1e-7 : (R)1e-12) * g.dx[d];
        const R r0 = fmax(x - cp_coord<R, 1>(g, d, c), tiny), r1 = fmax(cp_coord<R, 1>(g, d, c + 1) - x, tiny);
        w[0] = r1 * g.inv_dx[d];
        w[1] = r0 * g.inv_dx[d];
        dd[0] = -r0;
        dd[1] = r1;
    } else {
#pragma unroll
        for (int i = 0; i <= O; i++) {
            w[i] = ax.w[i];
            dd[i] = cp_coord<R, O>(g, d, c + i) - x;
        }
    }
}

template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(256) k_affine_gather(StepArgs<R> a) {
    __shared__ Scales S;
    __shared__ long long sh_l[32];
    __shared__ float sh_f[32];
    load_scales_musl(a, S);
    const size_t N = (size_t)a.g.nodec;
    const Particles<R> &P = a.P;
    const bool apic = (a.scheme == MPM_APIC);
    const R dmax[3] = {(OX == 2 ? (R)1.5 : (R)1) * a.g.dx[0], (OY == 2 ? (R)1.5 : (R)1) * a.g.dx[1],
                       (OZ == 2 ? (R)1.5 : (R)1) * a.g.dx[2]};
    long long gacc = 0;
    float bmax = 0.0f;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.num; p += (int64_t)gridDim.x * blockDim.x) {
        const R x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        const int cx = cell_of(x0, a.g, 0, oob), cy = cell_of(x1, a.g, 1, oob), cz = cell_of(x2, a.g, 2, oob);
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        axis_eval<R, OX>(x0, a.g, 0, cx, ax);
        axis_eval<R, OY>(x1, a.g, 1, cy, ay);
        axis_eval<R, OZ>(x2, a.g, 2, cz, az);
        R v[3] = {(R)0, (R)0, (R)0}, gu[3] = {(R)0, (R)0, (R)0};
        R B[9], D[6];   // D: xx yy zz xy xz yz
        R wx[OX + 1], wy[OY + 1], wz[OZ + 1], ex[OX + 1], ey[OY + 1], ez[OZ + 1];
        if (apic) {
            apic_axis<R, OX>(a.g, 0, cx, x0, ax, wx, ex);
            apic_axis<R, OY>(a.g, 1, cy, x1, ay, wy, ey);
            apic_axis<R, OZ>(a.g, 2, cz, x2, az, wz, ez);
        }
#pragma unroll
        for (int e = 0; e < 9; e++) B[e] = (R)0;
#pragma unroll
        for (int e = 0; e < 6; e++) D[e] = (R)0;
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R wxy = ax.w[i] * ay.w[j];
                    const R N_ = wxy * az.w[k];
                    const R g0 = ax.dw[i] * ay.w[j] * az.w[k], g1 = ax.w[i] * ay.dw[j] * az.w[k], g2 = wxy * az.dw[k];
                    const size_t gn = node_id(a.g, cx + i, cy + j, cz + k);
                    R G[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        G[c] = ld(a.G + c * N + gn);
                        v[c] += N_ * G[c];
                    }
                    const R e = ld(a.nei + gn);
                    gu[0] += g0 * e;
                    gu[1] += g1 * e;
                    gu[2] += g2 * e;
                    if (apic) {
                        const R d0 = ex[i], d1 = ey[j], d2 = ez[k], Na = wx[i] * wy[j] * wz[k];
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            const R NG = Na * G[c];
                            B[3 * c] += NG * d0;
                            B[3 * c + 1] += NG * d1;
                            B[3 * c + 2] += NG * d2;
                        }
                        D[0] += Na * d0 * d0;
                        D[1] += Na * d1 * d1;
                        D[2] += Na * d2 * d2;
                        D[3] += Na * d0 * d1;
                        D[4] += Na * d0 * d2;
                        D[5] += Na * d1 * d2;
                    } else {
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            B[3 * c] += g0 * G[c];
                            B[3 * c + 1] += g1 * G[c];
                            B[3 * c + 2] += g2 * G[c];
                        }
                    }
                }
        if (apic) {
            // A = B D^-1 with D^-1 = adj(D) / det(D) (D symmetric)
            const R c00 = D[1] * D[2] - D[5] * D[5], c01 = D[4] * D[5] - D[3] * D[2], c02 = D[3] * D[5] - D[4] * D[1];
            const R c11 = D[0] * D[2] - D[4] * D[4], c12 = D[4] * D[3] - D[0] * D[5], c22 = D[0] * D[1] - D[3] * D[3];
            const R det = D[0] * c00 + D[3] * c01 + D[4] * c02;
            const R id = (R)1 / det;
            const R Di[9] = {c00 * id, c01 * id, c02 * id, c01 * id, c11 * id, c12 * id, c02 * id, c12 * id, c22 * id};
            R Am[9];
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int jj = 0; jj < 3; jj++)
                    Am[3 * c + jj] = B[3 * c] * Di[jj] + B[3 * c + 1] * Di[3 + jj] + B[3 * c + 2] * Di[6 + jj];
#pragma unroll
            for (int e = 0; e < 9; e++) B[e] = Am[e];
        }
#pragma unroll
        for (int c = 0; c < 3; c++) P.v[c][p] = v[c];
#pragma unroll
        for (int e = 0; e < 9; e++) P.C[e][p] = B[e];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float bc = (float)(fabs(v[c]) + fabs(B[3 * c]) * dmax[0] + fabs(B[3 * c + 1]) * dmax[1] +
                                     fabs(B[3 * c + 2]) * dmax[2]);
            bmax = fmaxf(bmax, bc);
        }
        const R tv = (R)2 * ld(P.vol + p);
        const R h0 = gu[0] * tv, h1 = gu[1] * tv, h2 = gu[2] * tv;
        gacc += fx(h0 * h0 + h1 * h1 + h2 * h2, S.gd);
    }
    const long long gsum = block_reduce(gacc, OpAddL(), sh_l);
    const float bm = block_reduce(bmax, OpMaxF(), sh_f);
    if (threadIdx.x == 0) {
        if (gsum) atomicAdd(&a.ctl->geup_acc, (unsigned long long)gsum);
        if (bm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VMAX], bm * 1.000001f);
    }
}

// FP32 linear grids: the affine MUSL scatter as per-cell register sums (two
// threads per cell, thread h owns the four corners of z-layer h), the node
// pass of k_p2g_cell for the three momentum fields; a particle that left its
// sorted cell adds its own fixed-point atomics.
__global__ void __launch_bounds__(CELL_THREADS, 3) k_affine_musl_cell(StepArgs<float> a) {
    __shared__ float corner[3 * 8][BRC];
    __shared__ Scales S;
    const int b = blockIdx.x;
    const int lc = threadIdx.x >> 1, h = threadIdx.x & 1;
    const int *cs = a.cstart + (size_t)b * (BRC + 1);
    if (cs[0] == cs[BRC]) return;   // empty brick (uniform across the CTA)
    int ox, oy, oz;
    brick_origin(b, a.nbrick, ox, oy, oz);
    const int cx = ox + (lc % BRX), cy = oy + (lc / BRX) % BRY, cz = oz + lc / (BRX * BRY);
    load_scales_musl(a, S);
    const size_t N = (size_t)a.g.nodec;
    const Particles<float> &P = a.P;
    float acc[3][4];
#pragma unroll
    for (int f = 0; f < 3; f++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[f][c] = 0.0f;
    for (int p = cs[lc]; p < cs[lc + 1]; p++) {
        const float x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        const int px = cell_of(x0, a.g, 0, oob), py = cell_of(x1, a.g, 1, oob), pz = cell_of(x2, a.g, 2, oob);
        Axis<float, 1> ax, ay, az;
        axis_eval<float, 1>(x0, a.g, 0, px, ax);
        axis_eval<float, 1>(x1, a.g, 1, py, ay);
        axis_eval<float, 1>(x2, a.g, 2, pz, az);
        const float m = ld(P.m + p);
        const float v[3] = {ld(P.v[0] + p), ld(P.v[1] + p), ld(P.v[2] + p)};
        float A[9];
#pragma unroll
        for (int e = 0; e < 9; e++) A[e] = ld(P.C[e] + p);
        const bool mine = (px == cx) && (py == cy) && (pz == cz);
        const float wz = h ? az.w[1] : az.w[0], dz = cp_coord<float, 1>(a.g, 2, pz + h) - x2;
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const float Nm = ax.w[i] * ay.w[j] * wz * m;
                float vn[3];
                affine_velocity(v, A, cp_coord<float, 1>(a.g, 0, px + i) - x0, cp_coord<float, 1>(a.g, 1, py + j) - x1,
                                dz, vn);
                if (mine) {
#pragma unroll
                    for (int f = 0; f < 3; f++) acc[f][i + 2 * j] += Nm * vn[f];
                } else {
                    const size_t gn = node_id(a.g, px + i, py + j, pz + h);
#pragma unroll
                    for (int f = 0; f < 3; f++) atomic_add_i64(&a.acc2[f * N + gn], fx(Nm * vn[f], S.q));
                }
            }
    }
#pragma unroll
    for (int f = 0; f < 3; f++)
#pragma unroll
        for (int c = 0; c < 4; c++) corner[f * 8 + c + 4 * h][lc] = acc[f][c];
    __syncthreads();
    constexpr int NX = BRX + 1, NY = BRY + 1, NZ = BRZ + 1, NB = NX * NY * NZ;
    for (int it = threadIdx.x; it < NB * 3; it += CELL_THREADS) {
        const int f = it / NB, n = it % NB;
        const int nx = n % NX, ny = (n / NX) % NY, nz = n / (NX * NY);
        const int gx = ox + nx, gy = oy + ny, gz = oz + nz;
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        float sum = 0.0f;
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 2; j++)
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const int ex = nx - i, ey = ny - j, ez = nz - k;
                    if (ex >= 0 && ex < BRX && ey >= 0 && ey < BRY && ez >= 0 && ez < BRZ)
                        sum += corner[f * 8 + i + 2 * (j + 2 * k)][ex + BRX * (ey + BRY * ez)];
                }
        if (sum != 0.0f) atomic_add_i64(&a.acc2[(size_t)f * N + node_id(a.g, gx, gy, gz)], fx(sum, S.q));
    }
}

template <typename R>
__global__ void k_affine_scale(StepArgs<R> a) {
    a.ctl->sc_musl.q = make_fix(a.nump * a.mmax * (double)bits_f(a.ctl->nxt[a.parity ^ 1][B_VMAX]) * 1.0000001);
}

template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(256) k_affine_musl(StepArgs<R> a) {
    constexpr int BX = BRX + OX, BY = BRY + OY, BZ = BRZ + OZ, BOX = BX * BY * BZ;
    extern __shared__ unsigned long long sacc[];   // 3 * BOX
    __shared__ Scales S;
    if ((int)blockIdx.x >= *a.nwork) return;
    const WorkItem w = a.work[blockIdx.x];
    int ox, oy, oz;
    brick_origin(w.tile, a.nbrick, ox, oy, oz);
    for (int i = threadIdx.x; i < 3 * BOX; i += blockDim.x) sacc[i] = 0ull;
    load_scales_musl(a, S);
    const size_t N = (size_t)a.g.nodec;
    const Particles<R> &P = a.P;
    for (int p = w.begin + threadIdx.x; p < w.end; p += blockDim.x) {
        const R x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        const int cx = cell_of(x0, a.g, 0, oob), cy = cell_of(x1, a.g, 1, oob), cz = cell_of(x2, a.g, 2, oob);
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        axis_eval<R, OX>(x0, a.g, 0, cx, ax);
        axis_eval<R, OY>(x1, a.g, 1, cy, ay);
        axis_eval<R, OZ>(x2, a.g, 2, cz, az);
        const R m = ld(P.m + p);
        const R v[3] = {ld(P.v[0] + p), ld(P.v[1] + p), ld(P.v[2] + p)};
        R A[9];
#pragma unroll
        for (int e = 0; e < 9; e++) A[e] = ld(P.C[e] + p);
        const int lx = cx - ox, ly = cy - oy, lz = cz - oz;
        const bool in = (unsigned)lx < (unsigned)BRX && (unsigned)ly < (unsigned)BRY && (unsigned)lz < (unsigned)BRZ;
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R Nm = ax.w[i] * ay.w[j] * az.w[k] * m;
                    R vn[3];
                    affine_velocity(v, A, cp_coord<R, OX>(a.g, 0, cx + i) - x0, cp_coord<R, OY>(a.g, 1, cy + j) - x1,
                                    cp_coord<R, OZ>(a.g, 2, cz + k) - x2, vn);
                    const long long q0 = fx(Nm * vn[0], S.q), q1 = fx(Nm * vn[1], S.q), q2 = fx(Nm * vn[2], S.q);
                    if (in) {
                        const int li = (lx + i) + BX * ((ly + j) + BY * (lz + k));
                        atomic_add_i64(&sacc[li], q0);
                        atomic_add_i64(&sacc[BOX + li], q1);
                        atomic_add_i64(&sacc[2 * BOX + li], q2);
                    } else {
                        const size_t gn = node_id(a.g, cx + i, cy + j, cz + k);
                        atomic_add_i64(&a.acc2[gn], q0);
                        atomic_add_i64(&a.acc2[N + gn], q1);
                        atomic_add_i64(&a.acc2[2 * N + gn], q2);
                    }
                }
    }
    __syncthreads();
    for (int li = threadIdx.x; li < BOX; li += blockDim.x) {
        const int lx = li % BX, ly = (li / BX) % BY, lz = li / (BX * BY);
        const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        const size_t gn = node_id(a.g, gx, gy, gz);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            unsigned long long v = sacc[d * BOX + li];
            if (v) atomicAdd(&a.acc2[d * N + gn], v);
        }
    }
}

// ------------------------------------------------------------ grid pass 1
constexpr int GRID_THREADS = 256;                            // threads of a grid-pass CTA
constexpr int GRID_NPT = TILE * TILE * TILE / GRID_THREADS;  // nodes of a tile per thread
static_assert(GRID_NPT * GRID_THREADS == TILE * TILE * TILE, "a grid-pass CTA covers its tile exactly");

template <typename R, bool LIST>
__global__ void __launch_bounds__(GRID_THREADS) k_grid1(StepArgs<R> a) {
    pdl_wait();
    __shared__ double sh_d[32];
    __shared__ float sh_f[32];
    __shared__ bool s_last;
    __shared__ Scales S;
    float gmax = 0.0f, neimax = 0.0f;
    load_scales(a, S);
    const int ntl = LIST ? *a.ntlist : 1;
    for (int lt = LIST ? (int)blockIdx.x : 0; lt < ntl; lt += LIST ? (int)gridDim.x : 1) {
    const int t = LIST ? a.tlist[lt] : (int)blockIdx.x;
    float eu = 0.0f;
    const bool active = LIST || a.all_tiles || a.tileflag[t];
    if (active) {
        int tx, ty, tz;
        tile_coords(t, a.g.ntile, tx, ty, tz);
        const size_t N = (size_t)a.g.nodec;
        // the tile's nodes, GRID_NPT per thread: every load of them is issued
        // before any of them is used
        long long q[GRID_NPT][NACC];
        unsigned char bfl[GRID_NPT];
        double nvl[GRID_NPT];
        size_t nid[GRID_NPT];
        bool in[GRID_NPT];
#pragma unroll
        for (int k = 0; k < GRID_NPT; k++) {
            const int li = threadIdx.x + k * GRID_THREADS;
            const int gx = tx * TILE + (li % TILE), gy = ty * TILE + (li / TILE) % TILE, gz = tz * TILE + li / (TILE * TILE);
            in[k] = gx < a.g.nnc[0] && gy < a.g.nnc[1] && gz < a.g.nnc[2];
            nid[k] = in[k] ? node_id(a.g, gx, gy, gz) : 0;
            if (in[k]) {
#pragma unroll
                for (int f = 0; f < NACC; f++) q[k][f] = (long long)a.acc[f * N + nid[k]];
                bfl[k] = a.bcflag[nid[k]];
                nvl[k] = a.nvol[nid[k]];
            }
        }
#pragma unroll
        for (int k = 0; k < GRID_NPT; k++) {
            if (!in[k]) continue;
            const size_t n = nid[k];
            const R mass = unfx(q[k][0], S.m, (R)0);
            R vof = unfx(q[k][1], S.v, (R)0);
            R nv[3], na[3];
            const R im = (mass > a.mtol) ? recip<R>(mass) : (R)0;   // one reciprocal per node
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const R pc = unfx(q[k][2 + c], S.p, (R)0);
                const R fc = unfx(q[k][5 + c], S.f, (R)0);
                nv[c] = pc * im;
                na[c] = fc * im;
            }
            if (vof < a.mtol) vof = (R)0;
            const unsigned char bf = bfl[k];
            if (bf) {
#pragma unroll
                for (int c = 0; c < 3; c++)
                    if (bf & (1 << c)) {
                        nv[c] = a.bcval[c * N + n] * a.facl;   // BCSetVal
                        na[c] = (R)0;                           // BCSetZero
                    }
            }
            if (a.nvel_dl) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    a.nvel_dl[c * N + n] = nv[c];
                    a.naccel_dl[c * N + n] = na[c];
                }
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const R gv = (a.scheme == MPM_FLIP) ? na[c] : nv[c] + a.dt * na[c];
                a.G[c * N + n] = gv;
                gmax = fmaxf(gmax, fabsf((float)gv));
            }
            R e = vof - (R)nvl[k];
            e = e > (R)0 ? e : (R)0;
            a.nei[n] = e;
            eu += (float)e * (float)e;
            neimax = fmaxf(neimax, (float)e);
        }
    }
    // deterministic sum of nei^2: per-tile partials (by list position in list
    // mode), reduced in order by the last CTA
    double ebl = block_reduce((double)eu, OpAddD(), sh_d);
    if (threadIdx.x == 0) a.eu_part[LIST ? lt : t] = ebl;
    __syncthreads();
    }
    float gm = block_reduce(gmax, OpMaxF(), sh_f);
    float nm = block_reduce(neimax, OpMaxF(), sh_f);
    if (threadIdx.x == 0) {
        if (gm > 0.0f) atomic_max_pos(&a.ctl->cur[C_GMAX], gm * 1.000001f);
        if (nm > 0.0f) atomic_max_pos(&a.ctl->cur[C_NEIMAX], nm * 1.000001f);
        __threadfence();
        unsigned prev = atomicAdd(&a.ctl->tile_counter, 1u);
        s_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        double acc = 0.0;
        const int npart = LIST ? *a.ntlist : (int)gridDim.x;
        for (int i = threadIdx.x; i < npart; i += blockDim.x) acc += ((volatile double *)a.eu_part)[i];
        double tot = block_reduce(acc, OpAddD(), sh_d);
        if (threadIdx.x == 0) {
            a.ctl->eu_norm = tot;
            a.ctl->tile_counter = 0u;
            Scales sm;
            compute_scales(a, sm);
            a.ctl->sc_musl = sm;
        }
    }
}

// ------------------------------------------------------------ grid pass 2
template <typename R, bool LIST>
__global__ void __launch_bounds__(GRID_THREADS) k_grid2(StepArgs<R> a) {
    pdl_wait();
    __shared__ Scales S;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // b0 of DeltaCorrectionParticleShifting (material_point.cpp:219)
        double gd = (double)(long long)a.ctl->geup_acc * a.ctl->sc_musl.gd.inv;
        a.ctl->b0 = (!a.shifting || gd < (double)a.mtol) ? 0.0 : a.ctl->eu_norm / gd;
    }
    load_scales_musl(a, S);
    const int ntl = LIST ? *a.ntlist : 1;
    for (int lt = LIST ? (int)blockIdx.x : 0; lt < ntl; lt += LIST ? (int)gridDim.x : 1) {
    const int t = LIST ? a.tlist[lt] : (int)blockIdx.x;
    if (!(LIST || a.all_tiles || a.tileflag[t])) return;
    int tx, ty, tz;
    tile_coords(t, a.g.ntile, tx, ty, tz);
    const size_t N = (size_t)a.g.nodec;
    long long q[GRID_NPT][4];
    unsigned char bfl[GRID_NPT];
    size_t nid[GRID_NPT];
    bool in[GRID_NPT];
#pragma unroll
    for (int k = 0; k < GRID_NPT; k++) {
        const int li = threadIdx.x + k * GRID_THREADS;
        const int gx = tx * TILE + (li % TILE), gy = ty * TILE + (li / TILE) % TILE, gz = tz * TILE + li / (TILE * TILE);
        in[k] = gx < a.g.nnc[0] && gy < a.g.nnc[1] && gz < a.g.nnc[2];
        nid[k] = in[k] ? node_id(a.g, gx, gy, gz) : 0;
        if (in[k]) {
            q[k][0] = (long long)a.acc[nid[k]];
#pragma unroll
            for (int c = 0; c < 3; c++) q[k][1 + c] = (long long)a.acc2[c * N + nid[k]];
            bfl[k] = a.bcflag[nid[k]];
        }
    }
#pragma unroll
    for (int k = 0; k < GRID_NPT; k++) {
        if (!in[k]) continue;
        const size_t n = nid[k];
        const R mass = unfx(q[k][0], S.m, (R)0);
        R nv[3];
        const R im = (mass > a.mtol) ? recip<R>(mass) : (R)0;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const R pc = unfx(q[k][1 + c], S.q, (R)0);
            nv[c] = pc * im;
        }
        const unsigned char bf = bfl[k];
        if (bf) {
#pragma unroll
            for (int c = 0; c < 3; c++)
                if (bf & (1 << c)) nv[c] = a.bcval[c * N + n] * a.facl;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) a.nvel2[c * N + n] = nv[c];
        if (!a.all_tiles) {
#pragma unroll
            for (int f = 0; f < NACC; f++)
                if (!(a.fbar && f == 1)) a.acc[f * N + n] = 0ull;   // F-bar: k_fbar_grid reads nvof first
#pragma unroll
            for (int c = 0; c < 3; c++) a.acc2[c * N + n] = 0ull;
        }
    }
    if (!a.all_tiles) {
        __syncthreads();
        if (threadIdx.x == 0) a.tileflag[t] = 0;
    }
    }
}

// ================================================================= F-bar
// cal_def_grad_bar (module/solid/explicit/fbar_projection.cpp:18-93), after
// the MUSL nodal velocities (nvel2) are final:
//   k_fbar_trial    per particle the step's dF = I + dt grad(nvel2) (the
//                   update's own formula) and the trial J = Jbar det(dF),
//                   stored; records max(J vol)
//   k_fbar_scale    the fixed-point scale of the nodal sums from that bound
//   k_fbar_scatter  sum_p N J vol into the nodes (int64 fixed point)
//   k_fbar_grid     nJbar = sum / nvof (0 where nvof <= mtol) into the free
//                   gather field G; clears the sums and the nvof sums
// FP32 keeps J - 1 in place of J (trial, projected and gathered): the sums
// are of N (J - 1) vol, a node with nvof <= mtol holds -1 (its nJbar = 0),
// so sum_i N_i field_i = Jbar - 1 by the partition of unity.
// and the update kernel (FBAR) gathers Jbar, scales dF by cbrt(Jbar / J),
// advances def_grad_bar and hands (def_grad_bar, Jbar, scaled dF) to the
// stress models, the plain J to the volume (var_trans_solid_explicit.cpp:
// 176-180, 298-304).
template <typename R, int OX, int OY, int OZ>
__device__ __forceinline__ R fbar_trial_j(const StepArgs<R> &a, const Particles<R> &P, int64_t p, Axis<R, OX> &ax,
                                          Axis<R, OY> &ay, Axis<R, OZ> &az, int &cx, int &cy, int &cz) {
    const size_t N = (size_t)a.g.nodec;
    const R x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
    bool oob = false;
    cx = cell_of(x0, a.g, 0, oob);
    cy = cell_of(x1, a.g, 1, oob);
    cz = cell_of(x2, a.g, 2, oob);
    axis_eval<R, OX>(x0, a.g, 0, cx, ax);
    axis_eval<R, OY>(x1, a.g, 1, cy, ay);
    axis_eval<R, OZ>(x2, a.g, 2, cz, az);
    R D[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if constexpr (sizeof(R) == 4 && OX == 1 && OY == 1 && OZ == 1) {
        // FP32 linear: the update's tensor-product gather (the same dF)
        const size_t b0 = node_id(a.g, cx, cy, cz), sy = (size_t)a.g.nnc[0], sz = sy * (size_t)a.g.nnc[1];
        float V[2][2][2], val, g[3];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            tp_load(a.nvel2 + r * N, b0, sy, sz, V);
            tp_eval(V, ax, ay, az, val, g);
#pragma unroll
            for (int c = 0; c < 3; c++) D[r][c] = g[c] * a.dt;
        }
    } else {
#pragma unroll
    for (int k = 0; k <= OZ; k++)
#pragma unroll
        for (int j = 0; j <= OY; j++)
#pragma unroll
            for (int i = 0; i <= OX; i++) {
                const R wxy = ax.w[i] * ay.w[j];
                const R dn[3] = {ax.dw[i] * ay.w[j] * az.w[k], ax.w[i] * ay.dw[j] * az.w[k], wxy * az.dw[k]};
                const size_t gn = node_id(a.g, cx + i, cy + j, cz + k);
                const R nv[3] = {ld(a.nvel2 + gn), ld(a.nvel2 + N + gn), ld(a.nvel2 + 2 * N + gn)};
#pragma unroll
                for (int r = 0; r < 3; r++)
#pragma unroll
                    for (int c = 0; c < 3; c++) D[r][c] += dn[c] * nv[r] * a.dt;
            }
    }
    if constexpr (sizeof(R) == 8) {
#pragma unroll
        for (int r = 0; r < 3; r++) D[r][r] += (R)1;
        return ld(P.Jb + p) * det3(D);
    } else {
        // FP32 carries J - 1: (1 + jb)(1 + dm) - 1 without the rounding of numbers near 1
        const R jb = ld(P.Jb + p), dm = (R)det_ipm1((const float(*)[3])D);
        return jb + dm + jb * dm;
    }
}

template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(256) k_fbar_trial(StepArgs<R> a) {
    __shared__ float sh_f[32];
    const Particles<R> &P = a.P;
    float jvmax = 0.0f;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.num; p += (int64_t)gridDim.x * blockDim.x) {
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        int cx, cy, cz;
        const R jt = fbar_trial_j<R, OX, OY, OZ>(a, P, p, ax, ay, az, cx, cy, cz);
        P.Jt[p] = jt;
        jvmax = fmaxf(jvmax, (float)fabs(jt * ld(P.vol + p)));
    }
    const float m = block_reduce(jvmax, OpMaxF(), sh_f);
    if (threadIdx.x == 0 && m > 0.0f) atomic_max_pos(&a.ctl->cur[C_JVMAX], m * 1.000001f);
}

template <typename R>
__global__ void k_fbar_scale(StepArgs<R> a) {
    a.ctl->sc_fbar = make_fix(a.nump * (double)bits_f(a.ctl->cur[C_JVMAX]) * 1.0000001);
}

template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(256) k_fbar_scatter(StepArgs<R> a) {
    __shared__ Fix F;
    if (threadIdx.x == 0) F = a.ctl->sc_fbar;
    __syncthreads();
    const Particles<R> &P = a.P;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.num; p += (int64_t)gridDim.x * blockDim.x) {
        const R x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        const int cx = cell_of(x0, a.g, 0, oob), cy = cell_of(x1, a.g, 1, oob), cz = cell_of(x2, a.g, 2, oob);
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        axis_eval<R, OX>(x0, a.g, 0, cx, ax);
        axis_eval<R, OY>(x1, a.g, 1, cy, ay);
        axis_eval<R, OZ>(x2, a.g, 2, cz, az);
        const R jv = ld(P.Jt + p) * ld(P.vol + p);
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const long long q = fx(ax.w[i] * ay.w[j] * az.w[k] * jv, F);
                    if (q) atomic_add_i64(&a.facc[node_id(a.g, cx + i, cy + j, cz + k)], q);
                }
    }
}

// FP32 linear grids: the same projection as per-cell register sums (two
// threads per cell, thread h owns the four corners of z-layer h) and one
// fixed-point RED per node; a particle that left its sorted cell adds its own
// atomics.
__global__ void __launch_bounds__(CELL_THREADS, 3) k_fbar_scatter_cell(StepArgs<float> a) {
    __shared__ float corner[8][BRC];
    __shared__ Fix F;
    const int b = blockIdx.x;
    const int lc = threadIdx.x >> 1, h = threadIdx.x & 1;
    const int *cs = a.cstart + (size_t)b * (BRC + 1);
    if (cs[0] == cs[BRC]) return;   // empty brick (uniform across the CTA)
    if (threadIdx.x == 0) F = a.ctl->sc_fbar;
    int ox, oy, oz;
    brick_origin(b, a.nbrick, ox, oy, oz);
    const int cx = ox + (lc % BRX), cy = oy + (lc / BRX) % BRY, cz = oz + lc / (BRX * BRY);
    __syncthreads();
    const Particles<float> &P = a.P;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int p = cs[lc]; p < cs[lc + 1]; p++) {
        const float x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        const int px = cell_of(x0, a.g, 0, oob), py = cell_of(x1, a.g, 1, oob), pz = cell_of(x2, a.g, 2, oob);
        Axis<float, 1> ax, ay, az;
        axis_eval<float, 1>(x0, a.g, 0, px, ax);
        axis_eval<float, 1>(x1, a.g, 1, py, ay);
        axis_eval<float, 1>(x2, a.g, 2, pz, az);
        const float jv = ld(P.Jt + p) * ld(P.vol + p) * (h ? az.w[1] : az.w[0]);
        const bool mine = (px == cx) && (py == cy) && (pz == cz);
#pragma unroll
        for (int j = 0; j < 2; j++)
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const float q = ax.w[i] * ay.w[j] * jv;
                if (mine) {
                    acc[i + 2 * j] += q;
                } else {
                    const long long v = fx(q, F);
                    if (v) atomic_add_i64(&a.facc[node_id(a.g, px + i, py + j, pz + h)], v);
                }
            }
    }
#pragma unroll
    for (int c = 0; c < 4; c++) corner[c + 4 * h][lc] = acc[c];
    __syncthreads();
    constexpr int NX = BRX + 1, NY = BRY + 1, NZ = BRZ + 1, NB = NX * NY * NZ;
    for (int n = threadIdx.x; n < NB; n += CELL_THREADS) {
        const int nx = n % NX, ny = (n / NX) % NY, nz = n / (NX * NY);
        const int gx = ox + nx, gy = oy + ny, gz = oz + nz;
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        float sum = 0.0f;
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 2; j++)
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const int ex = nx - i, ey = ny - j, ez = nz - k;
                    if (ex >= 0 && ex < BRX && ey >= 0 && ey < BRY && ez >= 0 && ez < BRZ)
                        sum += corner[i + 2 * (j + 2 * k)][ex + BRX * (ey + BRY * ez)];
                }
        if (sum != 0.0f) atomic_add_i64(&a.facc[node_id(a.g, gx, gy, gz)], fx(sum, F));
    }
}

template <typename R, bool LIST>
__global__ void __launch_bounds__(256) k_fbar_grid(StepArgs<R> a) {
    __shared__ Scales S;
    __shared__ Fix F;
    load_scales(a, S);
    if (threadIdx.x == 0) F = a.ctl->sc_fbar;
    __syncthreads();
    const size_t N = (size_t)a.g.nodec;
    const int ntl = LIST ? *a.ntlist : 1;
    for (int lt = LIST ? (int)blockIdx.x : 0; lt < ntl; lt += LIST ? (int)gridDim.x : 1) {
        const int t = LIST ? a.tlist[lt] : (int)blockIdx.x;
        int tx, ty, tz;
        tile_coords(t, a.g.ntile, tx, ty, tz);
        for (int li = threadIdx.x; li < TILE * TILE * TILE; li += blockDim.x) {
            const int gx = tx * TILE + (li % TILE), gy = ty * TILE + (li / TILE) % TILE,
                      gz = tz * TILE + li / (TILE * TILE);
            if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
            const size_t n = node_id(a.g, gx, gy, gz);
            const R nvof = unfx((long long)a.acc[N + n], S.v, (R)0);
            const R nj = unfx((long long)a.facc[n], F, (R)0);
            a.G[n] = (nvof > a.mtol) ? nj / nvof : (sizeof(R) == 8 ? (R)0 : (R)-1);
            a.facc[n] = 0ull;
            if (!a.all_tiles) a.acc[N + n] = 0ull;
        }
    }
}

// Compaction of the active-tile flags into a list in tile order (one CTA).
__global__ void __launch_bounds__(1024) k_tile_list(const unsigned char *flag, int ntiles, int *list, int *nlist) {
    pdl_wait();
    __shared__ int s_cnt[1024];
    const int T = blockDim.x;
    const int per = (ntiles + T - 1) / T;
    const int lo = threadIdx.x * per, hi = min(lo + per, ntiles);
    int cnt = 0;
    for (int t = lo; t < hi; t++) cnt += flag[t] != 0;
    s_cnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int off = 1; off < T; off <<= 1) {
        const int v = threadIdx.x >= off ? s_cnt[threadIdx.x - off] : 0;
        __syncthreads();
        s_cnt[threadIdx.x] += v;
        __syncthreads();
    }
    int base = s_cnt[threadIdx.x] - cnt;
    for (int t = lo; t < hi; t++)
        if (flag[t]) list[base++] = t;
    if (threadIdx.x == T - 1) *nlist = s_cnt[T - 1];
}

// ----------------------------------------------- G2P 2: F, x, vol, stress
// One thread per particle (coalesced particle I/O; node gathers hit L1/L2).
template <typename R, int OX, int OY, int OZ, bool FBAR = false>
__global__ void __launch_bounds__(256) k_g2p_update(StepArgs<R> a) {
    __shared__ float sh_f[32];
    __shared__ int sh_i[32];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t N = (size_t)a.g.nodec;
    const Particles<R> &P = a.P;
    const R rb0 = (R)a.ctl->b0;
    float volmax = 0.0f, vsmax = 0.0f;
    int bad = 0;
    if (p < a.num) {
        R x[3] = {ld(P.x[0] + p), ld(P.x[1] + p), ld(P.x[2] + p)};
        bool oob = false;
        const int cx = cell_of(x[0], a.g, 0, oob), cy = cell_of(x[1], a.g, 1, oob), cz = cell_of(x[2], a.g, 2, oob);
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        axis_eval<R, OX>(x[0], a.g, 0, cx, ax);
        axis_eval<R, OY>(x[1], a.g, 1, cy, ay);
        axis_eval<R, OZ>(x[2], a.g, 2, cz, az);
        R D[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        R xn[3] = {x[0], x[1], x[2]};
        R du[3] = {(R)0, (R)0, (R)0};
        R gu[3] = {(R)0, (R)0, (R)0};
        R jbg = (R)0;   // F-bar: Jbar gathered from the projected nodal J
        constexpr bool FP64 = sizeof(R) == 8;
        if constexpr (!FP64 && OX == 1 && OY == 1 && OZ == 1) {
            // FP32 linear (the F-bar step): the tensor-product gather of the
            // staged update, from one base index
            const size_t b0 = node_id(a.g, cx, cy, cz), sy = (size_t)a.g.nnc[0], sz = sy * (size_t)a.g.nnc[1];
            float V[2][2][2], val, g[3];
#pragma unroll
            for (int r = 0; r < 3; r++) {
                tp_load(a.nvel2 + r * N, b0, sy, sz, V);
                tp_eval(V, ax, ay, az, val, g);
                du[r] = val;
#pragma unroll
                for (int c = 0; c < 3; c++) D[r][c] = g[c] * a.dt;
            }
            if (rb0 != (R)0) {
                tp_load(a.nei, b0, sy, sz, V);
                tp_eval(V, ax, ay, az, val, gu);
            }
            if constexpr (FBAR) {
                tp_load(a.G, b0, sy, sz, V);
                tp_eval(V, ax, ay, az, jbg, g);
            }
        } else {
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R wxy = ax.w[i] * ay.w[j];
                    const R N_ = wxy * az.w[k];
                    const R dn[3] = {ax.dw[i] * ay.w[j] * az.w[k], ax.w[i] * ay.dw[j] * az.w[k], wxy * az.dw[k]};
                    const size_t gn = node_id(a.g, cx + i, cy + j, cz + k);
                    const R nv[3] = {ld(a.nvel2 + gn), ld(a.nvel2 + N + gn), ld(a.nvel2 + 2 * N + gn)};
#pragma unroll
                    for (int r = 0; r < 3; r++)
#pragma unroll
                        for (int c = 0; c < 3; c++) D[r][c] += dn[c] * nv[r] * a.dt;
                    if (FP64) {
                        // FLIP::VarG2P on coord, term by term as the reference adds them
                        const R Nd = N_ * a.dt;
#pragma unroll
                        for (int c = 0; c < 3; c++) xn[c] += Nd * nv[c];
                    } else {
#pragma unroll
                        for (int c = 0; c < 3; c++) du[c] += N_ * nv[c];
                    }
                    if (rb0 != (R)0) {
                        const R e = ld(a.nei + gn);
#pragma unroll
                        for (int c = 0; c < 3; c++) gu[c] += dn[c] * e;
                    }
                    if constexpr (FBAR) jbg += N_ * ld(a.G + gn);
                }
        }
        if (!FP64) {
            // FP32: one rounding of the position per step
#pragma unroll
            for (int c = 0; c < 3; c++) xn[c] += du[c] * a.dt;
        }
        if (rb0 != (R)0) {
            const R tv = (R)2 * ld(P.vol + p);
#pragma unroll
            for (int c = 0; c < 3; c++) xn[c] += -rb0 * (gu[c] * tv);
        }
        // F <- (I + D) F  (var_trans_solid_explicit.cpp:276-290)
        R F[3][3], Fn[3][3];
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++) F[r][c] = ld(P.F[3 * r + c] + p);
        R Dm[3][3];   // delta_def_grad - I as the stress update sees it
        R J;
        if constexpr (FP64) {
            // FP64 keeps the reference's arithmetic: ddg = D + I, F = ddg F, deps = ddg_ii - 1
            R ddg[3][3];
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) ddg[r][c] = D[r][c] + (r == c ? (R)1 : (R)0);
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    R acc = (R)0;
#pragma unroll
                    for (int k2 = 0; k2 < 3; k2++) acc += ddg[r][k2] * F[k2][c];
                    Fn[r][c] = acc;
                    Dm[r][c] = (r == c) ? ddg[r][c] - (R)1 : ddg[r][c];
                }
            J = det3(Fn);
        } else {
            // FP32 stores H = F - I: H <- H + D + D H keeps the small strain exact to
            // FP32 rounding instead of to the rounding of numbers near 1
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    R acc = F[r][c] + D[r][c];
#pragma unroll
                    for (int k2 = 0; k2 < 3; k2++) acc += D[r][k2] * F[k2][c];
                    Fn[r][c] = acc;
                    Dm[r][c] = D[r][c];
                }
            J = (R)1 + (R)det_ipm1((const float(*)[3])Fn);
        }
        // the F the stress models see (def_grad_bar under F-bar) and the J in
        // the logarithm of the Neo-Hookean volumetric term (det_def_grad_bar)
        R Fs[3][3];
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++) Fs[r][c] = Fn[r][c];
        R jl = J;
        if constexpr (FBAR) {
            const R jt = ld(P.Jt + p);
            R Fb[3][3];
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) Fb[r][c] = ld(P.Fb[3 * r + c] + p);
            if constexpr (FP64) {
                const R sc = cbrt(jbg / jt);
                R dd[3][3];
#pragma unroll
                for (int r = 0; r < 3; r++)
#pragma unroll
                    for (int c = 0; c < 3; c++) dd[r][c] = (D[r][c] + (r == c ? (R)1 : (R)0)) * sc;
#pragma unroll
                for (int r = 0; r < 3; r++)
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        R acc = (R)0;
#pragma unroll
                        for (int k2 = 0; k2 < 3; k2++) acc += dd[r][k2] * Fb[k2][c];
                        Fs[r][c] = acc;
                        Dm[r][c] = (r == c) ? dd[r][c] - (R)1 : dd[r][c];
                    }
            } else {
                // FP32 (jbg, jt are J - 1): sc - 1 from log1p / expm1, H-form update of def_grad_bar
                const R sm1 = expm1f(log1pf((jbg - jt) / (1.0f + jt)) * (1.0f / 3.0f));
                const R sc = (R)1 + sm1;
                R Db[3][3];
#pragma unroll
                for (int r = 0; r < 3; r++)
#pragma unroll
                    for (int c = 0; c < 3; c++) Db[r][c] = sc * D[r][c] + (r == c ? sm1 : (R)0);
#pragma unroll
                for (int r = 0; r < 3; r++)
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        R acc = Fb[r][c] + Db[r][c];
#pragma unroll
                        for (int k2 = 0; k2 < 3; k2++) acc += Db[r][k2] * Fb[k2][c];
                        Fs[r][c] = acc;
                        Dm[r][c] = Db[r][c];
                    }
            }
            jl = jbg;
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) P.Fb[3 * r + c][p] = Fs[r][c];
            P.Jb[p] = jbg;
        }
        const R volp = J * ld(P.vol0 + p);
        R s[6];
#pragma unroll
        for (int k = 0; k < 6; k++) s[k] = ld(P.s[k] + p);
        const int mid = P.matid[p];
        const int model = a.iprop[mid];
        // FP32 reads the FP32 copy of the table (no FP64 loads and conversions per particle)
        auto mprop = [&](int k) -> R {
            if constexpr (sizeof(R) == 4) return a.matpropf[3 * mid + k];
            else return (R)a.matprop[3 * mid + k];
        };
        const R E = mprop(0), nu = mprop(1);
        if (model == 0) {
            lin_elast_update(s, Dm, E, nu);
        } else if (model == 1) {
            if constexpr (FBAR) {
                if constexpr (sizeof(R) == 8) neo_hookean_stress_bar(s, Fs, J, jl, E, nu);
                else neo_hookean_stress_h_bar(s, Fs, det_ipm1(Fn), jl, E, nu);   // jl = Jbar - 1
            } else {
                if constexpr (sizeof(R) == 8) neo_hookean_stress(s, Fn, J, E, nu);
                else neo_hookean_stress_h(s, Fn, det_ipm1(Fn), E, nu);
            }
        } else if (model == 2) {
            if constexpr (sizeof(R) == 8) stvk_stress(s, Fs, J, E, nu);
            else stvk_stress_h(s, Fs, det_ipm1(Fn), E, nu);
        } else if (model == 3) {   // mat_prop = {c1, c2, bulk}
            if constexpr (sizeof(R) == 8) mooney_rivlin_stress(s, Fs, J, E, nu, mprop(2));
            else mooney_rivlin_stress_h(s, Fs, det_ipm1(Fn), E, nu, mprop(2));
        } else if (model == 4) {
            R jm1;
            if constexpr (sizeof(R) == 8) jm1 = J - (R)1;
            else jm1 = det_ipm1(Fn);
            tait_stress<R>(s, Dm, jm1, ld(P.m + p) * recip<R>(ld(P.vol0 + p)), E, nu, mprop(2),
                           recip<R>(a.dt));
        } else if (model == -1) {
#pragma unroll
            for (int k = 0; k < 6; k++) s[k] = (R)0;
        }
        const bool fin = isfinite(xn[0]) && isfinite(xn[1]) && isfinite(xn[2]) && isfinite(J) && isfinite(s[0]) &&
                         isfinite(s[1]) && isfinite(s[2]) && isfinite(s[3]) && isfinite(s[4]) && isfinite(s[5]);
        bad += !fin;
#pragma unroll
        for (int c = 0; c < 3; c++) P.x[c][p] = xn[c];
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++) P.F[3 * r + c][p] = Fn[r][c];
#pragma unroll
        for (int k = 0; k < 6; k++) P.s[k][p] = s[k];
        P.vol[p] = volp;
        const float rs0 = fabsf((float)s[0]) + fabsf((float)s[5]) + fabsf((float)s[4]);
        const float rs1 = fabsf((float)s[5]) + fabsf((float)s[1]) + fabsf((float)s[3]);
        const float rs2 = fabsf((float)s[4]) + fabsf((float)s[3]) + fabsf((float)s[2]);
        const float vf = fabsf((float)volp);
        volmax = vf;
        vsmax = vf * fmaxf(rs0, fmaxf(rs1, rs2));
    }
    const float vm = block_reduce(volmax, OpMaxF(), sh_f);
    const float sm = block_reduce(vsmax, OpMaxF(), sh_f);
    const int nb = block_reduce(bad, OpAddI(), sh_i);
    if (threadIdx.x == 0) {
        if (vm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VOLMAX], vm * 1.000001f);
        if (sm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VOLSMAX], sm * 1.000001f);
        if (nb) atomicAdd(&a.ctl->err_nonfinite, (unsigned)nb);
    }
}

// ------------------------------------- G2P 2, FP32 linear, TMA-staged input
// The same update as k_g2p_update for FP32 and linear shape functions, with
// the particle fields it reads (x 3, H 9, sigma 6, vol0, vol, matid) brought
// into shared memory by bulk asynchronous copies, two chunks of UCH particles
// in flight per CTA, so that memory parallelism does not depend on how many
// warps are resident.  Persistent CTAs walk the chunks with a grid stride.
// Node values for the particle update: nvel2 (3 components) and nei.
struct GlobalNodes {
    const float *nvel2, *nei;
    size_t N;
    KGeom<float> g;
    __device__ __forceinline__ void get(int gx, int gy, int gz, bool shift, float *nv, float &e) const {
        const size_t gn = node_id(g, gx, gy, gz);
        nv[0] = ld(nvel2 + gn);
        nv[1] = ld(nvel2 + N + gn);
        nv[2] = ld(nvel2 + 2 * N + gn);
        if (shift) e = ld(nei + gn);
    }
};

// The same values from a brick's node box in shared memory, or from global
// memory for a particle whose cell lies outside the brick.
struct BoxNodes {
    const float *box;   // [4][NBX] : nvel2 x, y, z, nei
    int ox, oy, oz;
    GlobalNodes gl;
    static constexpr int NX = BRX + 1, NY = BRY + 1, NZ = BRZ + 1, NBX = NX * NY * NZ;
    __device__ __forceinline__ bool inside(int cx, int cy, int cz) const {
        return (unsigned)(cx - ox) < (unsigned)BRX && (unsigned)(cy - oy) < (unsigned)BRY &&
               (unsigned)(cz - oz) < (unsigned)BRZ;
    }
    __device__ __forceinline__ void get(int gx, int gy, int gz, bool shift, float *nv, float &e) const {
        const int l = (gx - ox) + NX * ((gy - oy) + NY * (gz - oz));
        nv[0] = box[l];
        nv[1] = box[NBX + l];
        nv[2] = box[2 * NBX + l];
        if (shift) e = box[3 * NBX + l];
    }
};

// Second G2P pass of one FP32 particle on linear shape functions
// (var_trans_solid_explicit.cpp:150-185, 247-296): F from the MUSL nodal
// velocities, position with shifting, volume and stress, written back.
// FLUIDJ: a Tait-fluid context, where field F[0] holds J - 1 (a separate
// instantiation, so that the solid kernels carry no fluid branch).
template <typename Nodes, bool FLUIDJ = false>
__device__ __forceinline__ void update_particle(const StepArgs<float> &a, const Particles<float> &P, int p,
                                                const float *x, const float (*H)[3], const float *s_in, float vol0,
                                                float volc, int mid, float rb0, const Nodes &nodes, float &volmax,
                                                float &vsmax, int &bad) {
    bool oob = false;
    const int cx = cell_of(x[0], a.g, 0, oob), cy = cell_of(x[1], a.g, 1, oob), cz = cell_of(x[2], a.g, 2, oob);
    Axis<float, 1> ax, ay, az;
    axis_eval<float, 1>(x[0], a.g, 0, cx, ax);
    axis_eval<float, 1>(x[1], a.g, 1, cy, ay);
    axis_eval<float, 1>(x[2], a.g, 2, cz, az);
    const bool shift = rb0 != 0.0f;
    // the cell's 8 nodes: V[q][k][j][i], q = nvel2 x, y, z and nei
    float V[4][2][2][2];
    if constexpr (std::is_same<Nodes, GlobalNodes>::value) {
        // one base index and the two strides instead of eight full index computations
        const size_t b0 = node_id(a.g, cx, cy, cz), sy = (size_t)a.g.nnc[0], sz = sy * (size_t)a.g.nnc[1];
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 2; j++)
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    const size_t gn = b0 + (size_t)i + (j ? sy : 0) + (k ? sz : 0);
                    V[0][k][j][i] = ld(nodes.nvel2 + gn);
                    V[1][k][j][i] = ld(nodes.nvel2 + nodes.N + gn);
                    V[2][k][j][i] = ld(nodes.nvel2 + 2 * nodes.N + gn);
                    V[3][k][j][i] = shift ? ld(nodes.nei + gn) : 0.0f;
                }
    } else {
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int j = 0; j < 2; j++)
#pragma unroll
                for (int i = 0; i < 2; i++) {
                    float nv[3], e = 0.0f;
                    nodes.get(cx + i, cy + j, cz + k, shift, nv, e);
                    V[0][k][j][i] = nv[0];
                    V[1][k][j][i] = nv[1];
                    V[2][k][j][i] = nv[2];
                    V[3][k][j][i] = e;
                }
    }
    // velocity, velocity gradient and shifting gradient (tp_eval)
    float val[4], grd[4][3];
#pragma unroll
    for (int q = 0; q < 3; q++) tp_eval(V[q], ax, ay, az, val[q], grd[q]);
    if (shift) tp_eval(V[3], ax, ay, az, val[3], grd[3]);
    else grd[3][0] = grd[3][1] = grd[3][2] = 0.0f;
    float D[3][3], du[3], gu[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        du[r] = val[r];
        gu[r] = grd[3][r];
#pragma unroll
        for (int c = 0; c < 3; c++) D[r][c] = grd[r][c] * a.dt;
    }
    float xn[3];
#pragma unroll
    for (int c = 0; c < 3; c++) xn[c] = x[c] + du[c] * a.dt;
    if (shift) {
        const float tv = 2.0f * volc;
#pragma unroll
        for (int c = 0; c < 3; c++) xn[c] += -rb0 * (gu[c] * tv);
    }
    float s[6];
#pragma unroll
    for (int k = 0; k < 6; k++) s[k] = s_in[k];
    const int model = a.iprop[mid];
    const float E = a.matpropf[3 * mid], nu = a.matpropf[3 * mid + 1];
    if constexpr (FLUIDJ) {
        // Tait fluid: only J is tracked, J_new - 1 = (1 + (J - 1)) det(I + D) - 1
        const float dj = det_ipm1(D);
        const float jm1 = H[0][0] + dj + H[0][0] * dj;
        const float J = 1.0f + jm1;
        const float volp = J * vol0;
        tait_stress<float>(s, D, jm1, P.m[p] * rcp_approx(vol0), E, nu, a.matpropf[3 * mid + 2],
                           rcp_approx(a.dt));
        const bool fin = isfinite(xn[0]) && isfinite(xn[1]) && isfinite(xn[2]) && isfinite(J) && isfinite(s[0]) &&
                         isfinite(s[1]) && isfinite(s[2]) && isfinite(s[3]) && isfinite(s[4]) && isfinite(s[5]);
        bad += !fin;
#pragma unroll
        for (int c = 0; c < 3; c++) P.x[c][p] = xn[c];
        P.F[0][p] = jm1;
#pragma unroll
        for (int k = 0; k < 6; k++) P.s[k][p] = s[k];
        P.vol[p] = volp;
        const float rs0 = fabsf(s[0]) + fabsf(s[5]) + fabsf(s[4]);
        const float rs1 = fabsf(s[5]) + fabsf(s[1]) + fabsf(s[3]);
        const float rs2 = fabsf(s[4]) + fabsf(s[3]) + fabsf(s[2]);
        const float vf = fabsf(volp);
        volmax = fmaxf(volmax, vf);
        vsmax = fmaxf(vsmax, vf * fmaxf(rs0, fmaxf(rs1, rs2)));
        return;
    }
    // H <- H + D + D H (the FP32 path stores H = F - I)
    float Hn[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float acc = H[r][c] + D[r][c];
#pragma unroll
            for (int k2 = 0; k2 < 3; k2++) acc += D[r][k2] * H[k2][c];
            Hn[r][c] = acc;
        }
    const float jm1 = det_ipm1(Hn);
    const float J = 1.0f + jm1;
    const float volp = J * vol0;
    if (model == 0) lin_elast_update(s, D, E, nu);
    else if (model == 1) neo_hookean_stress_h(s, Hn, jm1, E, nu);
    else if (model == 2) stvk_stress_h(s, Hn, jm1, E, nu);
    else if (model == 3) mooney_rivlin_stress_h(s, Hn, jm1, E, nu, a.matpropf[3 * mid + 2]);
    else if (model == 4)
        tait_stress<float>(s, D, jm1, P.m[p] * rcp_approx(vol0), E, nu, a.matpropf[3 * mid + 2],
                           rcp_approx(a.dt));
    else if (model == -1)
#pragma unroll
        for (int k = 0; k < 6; k++) s[k] = 0.0f;
    const bool fin = isfinite(xn[0]) && isfinite(xn[1]) && isfinite(xn[2]) && isfinite(J) && isfinite(s[0]) &&
                     isfinite(s[1]) && isfinite(s[2]) && isfinite(s[3]) && isfinite(s[4]) && isfinite(s[5]);
    bad += !fin;
#pragma unroll
    for (int c = 0; c < 3; c++) P.x[c][p] = xn[c];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) P.F[3 * r + c][p] = Hn[r][c];
#pragma unroll
    for (int k = 0; k < 6; k++) P.s[k][p] = s[k];
    P.vol[p] = volp;
    const float rs0 = fabsf(s[0]) + fabsf(s[5]) + fabsf(s[4]);
    const float rs1 = fabsf(s[5]) + fabsf(s[1]) + fabsf(s[3]);
    const float rs2 = fabsf(s[4]) + fabsf(s[3]) + fabsf(s[2]);
    const float vf = fabsf(volp);
    volmax = fmaxf(volmax, vf);
    vsmax = fmaxf(vsmax, vf * fmaxf(rs0, fmaxf(rs1, rs2)));
}

// Particle update, one CTA per brick: the brick's node box (nvel2, nei) is
// loaded into shared memory once, then the brick's particles (a contiguous
// range) are updated one per thread with coalesced loads and stores.
__global__ void __launch_bounds__(256) k_g2p_update_brick(StepArgs<float> a) {
    constexpr int NBX = BoxNodes::NBX;
    __shared__ float box[4 * NBX];
    __shared__ float sh_f[32];
    __shared__ int sh_i[32];
    const int b = blockIdx.x;
    const int *cs = a.cstart + (size_t)b * (BRC + 1);
    const int P0 = cs[0], P1 = cs[BRC];
    if (P0 == P1) return;
    const size_t N = (size_t)a.g.nodec;
    BoxNodes nodes;
    brick_origin(b, a.nbrick, nodes.ox, nodes.oy, nodes.oz);
    nodes.box = box;
    nodes.gl = GlobalNodes{a.nvel2, a.nei, N, a.g};
    const float rb0 = (float)a.ctl->b0;
    for (int l = threadIdx.x; l < NBX; l += blockDim.x) {
        const int nx = l % BoxNodes::NX, ny = (l / BoxNodes::NX) % BoxNodes::NY, nz = l / (BoxNodes::NX * BoxNodes::NY);
        const int gx = min(nodes.ox + nx, a.g.nnc[0] - 1), gy = min(nodes.oy + ny, a.g.nnc[1] - 1),
                  gz = min(nodes.oz + nz, a.g.nnc[2] - 1);
        const size_t gn = node_id(a.g, gx, gy, gz);
        box[l] = ld(a.nvel2 + gn);
        box[NBX + l] = ld(a.nvel2 + N + gn);
        box[2 * NBX + l] = ld(a.nvel2 + 2 * N + gn);
        box[3 * NBX + l] = rb0 != 0.0f ? ld(a.nei + gn) : 0.0f;
    }
    __syncthreads();
    const Particles<float> &P = a.P;
    float volmax = 0.0f, vsmax = 0.0f;
    int bad = 0;
    for (int p = P0 + threadIdx.x; p < P1; p += blockDim.x) {
        float x[3] = {ld(P.x[0] + p), ld(P.x[1] + p), ld(P.x[2] + p)};
        float H[3][3];
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++) H[r][c] = (a.fluidj && (r | c)) ? 0.0f : ld(P.F[3 * r + c] + p);
        float s6[6];
#pragma unroll
        for (int k = 0; k < 6; k++) s6[k] = ld(P.s[k] + p);
        bool oob = false;
        const int cx = cell_of(x[0], a.g, 0, oob), cy = cell_of(x[1], a.g, 1, oob), cz = cell_of(x[2], a.g, 2, oob);
        if (nodes.inside(cx, cy, cz))
            a.fluidj ? update_particle<BoxNodes, true>(a, P, p, x, H, s6, ld(P.vol0 + p), ld(P.vol + p), P.matid[p],
                                                       rb0, nodes, volmax, vsmax, bad)
                     : update_particle<BoxNodes>(a, P, p, x, H, s6, ld(P.vol0 + p), ld(P.vol + p), P.matid[p], rb0,
                                                 nodes, volmax, vsmax, bad);
        else
            a.fluidj ? update_particle<GlobalNodes, true>(a, P, p, x, H, s6, ld(P.vol0 + p), ld(P.vol + p),
                                                          P.matid[p], rb0, nodes.gl, volmax, vsmax, bad)
                     : update_particle<GlobalNodes>(a, P, p, x, H, s6, ld(P.vol0 + p), ld(P.vol + p), P.matid[p],
                                                    rb0, nodes.gl, volmax, vsmax, bad);
    }
    const float vm = block_reduce(volmax, OpMaxF(), sh_f);
    const float sm = block_reduce(vsmax, OpMaxF(), sh_f);
    const int nb = block_reduce(bad, OpAddI(), sh_i);
    if (threadIdx.x == 0) {
        if (vm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VOLMAX], vm * 1.000001f);
        if (sm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VOLSMAX], sm * 1.000001f);
        if (nb) atomicAdd(&a.ctl->err_nonfinite, (unsigned)nb);
    }
}

constexpr int UCH = 256;                          // particles per chunk (= threads per CTA)
constexpr int UNF = 20;                           // staged real fields
constexpr size_t USTAGE = (size_t)UNF * UCH * 4 + UCH * 4;   // bytes per stage
constexpr unsigned UWAIT = 1u << 22;              // bounded mbarrier wait (try_wait iterations)

// At most 80 registers, so that three CTAs (24 warps) are resident per SM.
template <bool FLUIDJ>
__global__ void __launch_bounds__(UCH, 3) k_g2p_update_tma(StepArgs<float> a, int nchunks) {
    pdl_wait();
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) unsigned long long bar[2];
    __shared__ float sh_f[32];
    __shared__ int sh_i[32];
    const size_t N = (size_t)a.g.nodec;
    const Particles<float> &P = a.P;
    const float *src[UNF] = {P.x[0], P.x[1], P.x[2], P.F[0], P.F[1], P.F[2], P.F[3], P.F[4], P.F[5], P.F[6],
                             P.F[7], P.F[8], P.s[0], P.s[1], P.s[2], P.s[3], P.s[4], P.s[5], P.vol0, P.vol};
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    // fields a step does not read are not copied: the previous stress unless
    // a material updates it incrementally, the current volume unless the
    // shifting is on (b0 != 0), the material ids of a one-material scene
    const float rb0 = (float)a.ctl->b0;
    const bool need_s = a.sigma_in != 0, need_vol = rb0 != 0.0f, need_mid = a.single_mat == 0;
    // a Tait-fluid context reads J - 1 (field 3) and none of the other eight F fields
    constexpr bool fluidj = FLUIDJ;
    auto wanted = [&](int f) {
        return (f < 12 || f >= 18 || need_s) && (f != 19 || need_vol) && !(fluidj && f >= 4 && f < 12);
    };
    // chunk k of the walk is particle chunk nchunks - 1 - k when the walk is reversed
    auto phys = [&](int k) { return a.rev_upd ? nchunks - 1 - k : k; };
    auto issue = [&](int chunk, int stage) {
        const int p0 = phys(chunk) * UCH;
        const int cnt = min(UCH, (int)a.num - p0);
        const unsigned bytes = (unsigned)((cnt + 3) & ~3) * 4u;   // whole 16-byte units (arrays are padded)
        float *dst = (float *)(smem + stage * USTAGE);
        unsigned nf = need_mid ? 1u : 0u;
        for (int f = 0; f < UNF; f++) nf += wanted(f) ? 1u : 0u;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bar[stage], bytes * nf);
        for (int f = 0; f < UNF; f++)
            if (wanted(f)) bulk_g2s(dst + f * UCH, src[f] + p0, bytes, &bar[stage]);
        if (need_mid) bulk_g2s(dst + UNF * UCH, P.matid + p0, bytes, &bar[stage]);
    };
    float volmax = 0.0f, vsmax = 0.0f;
    int bad = 0;
    bool failed = false;
    int it = 0;
    if (threadIdx.x == 0 && (int)blockIdx.x < nchunks) issue(blockIdx.x, 0);
    for (int chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x, it++) {
        const int stage = it & 1;
        if (threadIdx.x == 0 && chunk + (int)gridDim.x < nchunks) issue(chunk + gridDim.x, stage ^ 1);
        const bool ok = mbar_wait_bounded(&bar[stage], (unsigned)((it >> 1) & 1), UWAIT);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        const float *sf = (const float *)(smem + stage * USTAGE);
        const int *smid = (const int *)(sf + UNF * UCH);
        const int t = threadIdx.x;
        const int p = phys(chunk) * UCH + t;
        if (p < a.num) {
            float x[3] = {sf[0 * UCH + t], sf[1 * UCH + t], sf[2 * UCH + t]};
            float H[3][3];
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) H[r][c] = (fluidj && (r | c)) ? 0.0f : sf[(3 + 3 * r + c) * UCH + t];
            float s6[6];
#pragma unroll
            for (int k = 0; k < 6; k++) s6[k] = need_s ? sf[(12 + k) * UCH + t] : 0.0f;
            GlobalNodes gnodes{a.nvel2, a.nei, N, a.g};
            update_particle<GlobalNodes, FLUIDJ>(a, P, p, x, H, s6, sf[18 * UCH + t], need_vol ? sf[19 * UCH + t] : 0.0f,
                            need_mid ? smid[t] : 0, rb0, gnodes, volmax, vsmax, bad);
        }
        __syncthreads();   // the stage is refilled only after every thread has read it
    }
    if (failed) {
        // let the copies this CTA started land before the CTA exits
        if (threadIdx.x == 0) {
            atomicAdd(&a.ctl->err_timeout, 1u);
            const int stage = it & 1;
            mbar_wait_bounded(&bar[stage], (unsigned)((it >> 1) & 1), UWAIT);
            if (blockIdx.x + (it + 1) * gridDim.x < (unsigned)nchunks)
                mbar_wait_bounded(&bar[stage ^ 1], (unsigned)(((it + 1) >> 1) & 1), UWAIT);
        }
        __syncthreads();
        return;
    }
    const float vm = block_reduce(volmax, OpMaxF(), sh_f);
    const float sm = block_reduce(vsmax, OpMaxF(), sh_f);
    const int nb = block_reduce(bad, OpAddI(), sh_i);
    if (threadIdx.x == 0) {
        if (vm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VOLMAX], vm * 1.000001f);
        if (sm > 0.0f) atomic_max_pos(&a.ctl->nxt[a.parity ^ 1][B_VOLSMAX], sm * 1.000001f);
        if (nb) atomicAdd(&a.ctl->err_nonfinite, (unsigned)nb);
    }
}

// ------------------------------------------------------------- host side
template <typename R>
static StepArgs<R> make_args(mpm_ctx *c) {
    StepArgs<R> a;
    memset(&a, 0, sizeof(a));
    for (int d = 0; d < 3; d++) {
        a.g.xmin[d] = (R)c->g.xmin[d];
        a.g.dx[d] = (R)c->g.dx[d];
        a.g.inv_dx[d] = (R)(1.0 / c->g.dx[d]);
        a.g.nel[d] = c->g.nel[d];
        a.g.nnc[d] = c->g.nnc[d];
        a.g.ntile[d] = c->g.ntile[d];
        a.nbrick[d] = c->g.nbrick[d];
        a.grav[d] = (R)c->gravity[d];
    }
    a.g.nodec = c->g.nodec;
    a.num = c->num;
    char *base = (char *)c->pbuf[c->cur];
    size_t n = c->pstride, rs = sizeof(R);
    R *f = (R *)base;
    for (int k = 0; k < 3; k++) a.P.x[k] = f + (0 + k) * n;
    for (int k = 0; k < 3; k++) a.P.v[k] = f + (3 + k) * n;
    for (int k = 0; k < 9; k++) a.P.F[k] = f + (6 + k) * n;
    for (int k = 0; k < 6; k++) a.P.s[k] = f + (15 + k) * n;
    a.P.m = f + 21 * n;
    a.P.vol0 = f + 22 * n;
    a.P.vol = f + 23 * n;
    for (int k = 0; k < 3; k++) a.P.a[k] = c->nreal == 27 ? f + (24 + k) * n : nullptr;
    for (int k = 0; k < 9; k++) a.P.C[k] = c->affine ? f + (24 + k) * n : nullptr;
    for (int k = 0; k < 9; k++) a.P.Fb[k] = c->fbar ? f + (c->off_fbar + k) * n : nullptr;
    a.P.Jb = c->fbar ? f + (c->off_fbar + 9) * n : nullptr;
    a.P.Jt = c->fbar ? f + (c->off_fbar + 10) * n : nullptr;
    a.facc = c->d_facc;
    a.fbar = c->fbar ? 1 : 0;
    a.P.matid = (int *)(base + (size_t)c->nreal * n * rs);
    a.P.pid = a.P.matid + n;
    a.work = c->d_work;
    a.nwork = c->d_nwork;
    a.cstart = c->d_cstart;
    a.miss = c->d_tmp;
    a.blist = c->d_blist;
    a.nblist = c->d_nblist;
    a.tlist = c->d_tlist;
    a.ntlist = c->d_ntlist;
    a.acc = c->d_acc;
    a.acc2 = c->d_acc2;
    R *nod = (R *)c->d_nodal;
    size_t N = (size_t)c->g.nodec;
    a.G = nod;
    a.nei = nod + 3 * N;
    a.nvel2 = nod + 4 * N;
    a.nvel_dl = c->write_nodal_dl ? nod + 7 * N : nullptr;
    a.naccel_dl = c->write_nodal_dl ? nod + 10 * N : nullptr;
    a.nvol = c->d_nvol;
    a.bcflag = c->d_bcflag;
    a.bcval = (const R *)c->d_bcval;
    a.tileflag = c->d_tileflag;
    a.eu_part = c->d_eu_part;
    a.ctl = c->d_ctl;
    a.iprop = c->d_iprop;
    a.matprop = c->d_matprop;
    a.matpropf = c->d_matpropf;
    a.dt = (R)c->dt;
    a.facl = (R)c->facl;
    a.mtol = (R)c->mtol;
    a.parity = (int)(c->step & 1);
    a.scheme = c->scheme;
    a.shifting = c->shifting;
    a.all_tiles = c->write_nodal_dl ? 1 : 0;
    a.gnorm = c->gather_norm;
    a.sigma_in = c->sigma_in ? 1 : 0;
    a.single_mat = c->nmat == 1 ? 1 : 0;
    a.fluidj = c->fluid_j ? 1 : 0;
    if (c->alternate) {
        a.rev_p2g = a.rev_upd = a.parity;
        a.rev_g2p = a.parity ^ 1;
    }
    a.implicit = c->nreal == 27 ? 1 : 0;
    a.nump = (double)c->num;
    a.mmax = c->mmax;
    double gs = 0.0, gsum = 0.0;
    for (int d = 0; d < 3; d++) {
        double inv = 1.0 / c->g.dx[d];
        gs = fmax(gs, (c->g.order[d] == 2 ? 4.0 : 1.0) * inv);
        gsum = fmax(gsum, (c->g.order[d] == 2 ? 12.0 : 2.0) * inv);
    }
    a.gshape = gs;
    a.gsum = gsum;
    return a;
}

static bool use_cell_kernels(const mpm_ctx *c) {
    // the per-cell kernels carry the explicit fields only (no particle acceleration of the implicit solid)
    return c->cell_scatter && !c->affine && c->precision == 32 && c->nreal != 27 && c->g.order[0] == 1 &&
           c->g.order[1] == 1 && c->g.order[2] == 1;
}

static int num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 148;
    }
    return n;
}

// A launch of kernel k on st; with pdl, with programmatic stream
// serialization, so that its CTAs are scheduled while its predecessor drains
// (the kernel's pdl_wait orders its memory accesses after the predecessor).
template <typename... P, typename... A>
static void launch(bool pdl, void (*k)(P...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                   A... args) {
    if (!pdl) {
        k<<<grid, block, smem, st>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}

// persistent grid over the active-brick list: never more CTAs than bricks
static int list_grid(const mpm_ctx *c, int per_sm) {
    return std::min(c->g.nbricks, per_sm * num_sms());
}

// which: 0 P2G, 1 G2P + MUSL, 2 G2P update
template <typename R, int OX, int OY, int OZ>
static mpm_status launch_particle_kernel(mpm_ctx *c, int which) {
    StepArgs<R> a = make_args<R>(c);
    constexpr int BOX = (BRX + OX) * (BRY + OY) * (BRZ + OZ);
    if (c->num == 0) return MPM_OK;
    if (which == 0) {
        launch(c->pdl != 0, k_step_reset<R>, 1, 1, 0, c->stream, a);
        c->launches++;
        timer_begin(c, K_P2G);
        if constexpr (sizeof(R) == 4 && OX == 1 && OY == 1 && OZ == 1) {
            if (use_cell_kernels(c)) {
                if (c->tune.p2g_moments == 3) {
                    k_p2g_brick<<<c->g.nbricks, BCH, 0, c->stream>>>(a);
                } else if (c->tune.p2g_moments == 2) {
                    k_p2g_cell_mom<1, false><<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                } else if (c->tune.p2g_moments == 4) {
                    k_p2g_cell_mom<3, true><<<list_grid(c, 3), CELL_THREADS, 0, c->stream>>>(a);
                } else if (c->tune.p2g_moments == 5) {
                    k_p2g_cell_mom<2, true, true><<<list_grid(c, 2), CELL_THREADS, 0, c->stream>>>(a);
                } else if (c->tune.p2g_moments == 6) {
                    k_p2g_cell_mom<1, true, true><<<list_grid(c, 1), CELL_THREADS, 0, c->stream>>>(a);
                } else if (c->tune.p2g_moments) {
                    if (c->tune.brick_list)
                        launch(c->pdl != 0, k_p2g_cell_mom<2, true>, list_grid(c, 2), CELL_THREADS, 0, c->stream, a);
                    else
                        k_p2g_cell_mom<2, false><<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                } else if (c->tune.p2g_staged) {
                    static bool attr = false;
                    if (!attr) {
                        cudaFuncSetAttribute(k_p2g_cell_staged<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(2 * PSTAGE));
                        attr = true;
                    }
                    k_p2g_cell_staged<2><<<c->g.nbricks, CELL_THREADS, 2 * PSTAGE, c->stream>>>(a);
                } else if (c->tune.p2g_minb == 3) {
                    k_p2g_cell<3><<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                } else {
                    k_p2g_cell<2><<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                }
                launch(c->pdl != 0, k_p2g_misses<false>, 2 * num_sms(), 256, 0, c->stream, a);
                timer_end(c, K_P2G);
                c->launches += 2;
                return check_launch(c);
            }
        }
        if constexpr (sizeof(R) == 4 && OX == 1 && OY == 1 && OZ == 1) {
            if (c->affine && c->cell_scatter) {
                // TPIC / APIC: per-cell register sums with the affine momentum
                k_p2g_cell<2, true><<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                k_p2g_misses<true><<<2 * num_sms(), 256, 0, c->stream>>>(a);
                timer_end(c, K_P2G);
                c->launches += 2;
                return check_launch(c);
            }
        }
        size_t smem = (size_t)NACC * BOX * sizeof(unsigned long long);
        if (c->affine) {
            cudaFuncSetAttribute(k_p2g_box<R, OX, OY, OZ, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
            k_p2g_box<R, OX, OY, OZ, true><<<c->nwork_cap, 256, smem, c->stream>>>(a);
        } else {
            cudaFuncSetAttribute(k_p2g_box<R, OX, OY, OZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_p2g_box<R, OX, OY, OZ><<<c->nwork_cap, 256, smem, c->stream>>>(a);
        }
        timer_end(c, K_P2G);
    } else if (which == 1) {
        timer_begin(c, K_G2P_MUSL);
        if constexpr (sizeof(R) == 4 && OX == 1 && OY == 1 && OZ == 1) {
            if (use_cell_kernels(c)) {
                if (c->tune.musl_moments == 2) {
                    launch(c->pdl != 0, k_g2p_musl_mom<2, true>, list_grid(c, 2), CELL_THREADS, 0, c->stream, a);
                } else if (c->tune.musl_moments) {
                    k_g2p_musl_mom<3, true><<<list_grid(c, 3), CELL_THREADS, 0, c->stream>>>(a);
                } else if (c->tune.musl_staged == 2) {
                    k_musl_brick<<<c->g.nbricks, BCH, 0, c->stream>>>(a);
                } else if (c->tune.musl_staged) {
                    static bool attr = false;
                    if (!attr) {
                        cudaFuncSetAttribute(k_g2p_musl_cell_staged<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(2 * MSTAGE));
                        attr = true;
                    }
                    k_g2p_musl_cell_staged<3><<<c->g.nbricks, CELL_THREADS, 2 * MSTAGE, c->stream>>>(a);
                } else if (c->tune.musl_minb == 2) {
                    k_g2p_musl_cell<2, false><<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                } else if (c->tune.musl_minb == 5) {
                    k_g2p_musl_cell<4, true><<<list_grid(c, 4), CELL_THREADS, 0, c->stream>>>(a);
                } else if (c->tune.brick_list) {
                    k_g2p_musl_cell<3, true><<<list_grid(c, 3), CELL_THREADS, 0, c->stream>>>(a);
                } else {
                    k_g2p_musl_cell<3, false><<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                }
                launch(c->pdl != 0, k_musl_misses, 2 * num_sms(), 256, 0, c->stream, a);
                timer_end(c, K_G2P_MUSL);
                c->launches += 2;
                return check_launch(c);
            }
        }
        size_t smem = (size_t)3 * BOX * sizeof(unsigned long long);
        if (c->affine) {
            const int nb = (int)std::min<int64_t>((c->num + 255) / 256, 8 * num_sms());
            k_affine_gather<R, OX, OY, OZ><<<nb, 256, 0, c->stream>>>(a);
            k_affine_scale<R><<<1, 1, 0, c->stream>>>(a);
            bool cell = false;
            if constexpr (sizeof(R) == 4 && OX == 1 && OY == 1 && OZ == 1) {
                if (c->cell_scatter) {
                    k_affine_musl_cell<<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                    cell = true;
                }
            }
            if (!cell) {
                cudaFuncSetAttribute(k_affine_musl<R, OX, OY, OZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
                k_affine_musl<R, OX, OY, OZ><<<c->nwork_cap, 256, smem, c->stream>>>(a);
            }
            c->launches += 2;
        } else {
            cudaFuncSetAttribute(k_g2p_musl_box<R, OX, OY, OZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
            k_g2p_musl_box<R, OX, OY, OZ><<<c->nwork_cap, 256, smem, c->stream>>>(a);
        }
        timer_end(c, K_G2P_MUSL);
    } else {
        timer_begin(c, K_G2P_UPDATE);
        if (c->fbar) {
            const int nb = (int)((c->num + 255) / 256);
            const int pg = (int)std::min<int64_t>(nb, 8 * num_sms());
            k_fbar_trial<R, OX, OY, OZ><<<pg, 256, 0, c->stream>>>(a);
            k_fbar_scale<R><<<1, 1, 0, c->stream>>>(a);
            bool cell = false;
            if constexpr (sizeof(R) == 4 && OX == 1 && OY == 1 && OZ == 1) {
                if (c->cell_scatter) {
                    k_fbar_scatter_cell<<<c->g.nbricks, CELL_THREADS, 0, c->stream>>>(a);
                    cell = true;
                }
            }
            if (!cell) k_fbar_scatter<R, OX, OY, OZ><<<pg, 256, 0, c->stream>>>(a);
            if (!a.all_tiles)
                k_fbar_grid<R, true><<<std::min(c->g.ntiles, 6 * num_sms()), 256, 0, c->stream>>>(a);
            else
                k_fbar_grid<R, false><<<c->g.ntiles, 256, 0, c->stream>>>(a);
            k_g2p_update<R, OX, OY, OZ, true><<<nb, 256, 0, c->stream>>>(a);
            c->launches += 5;
            timer_end(c, K_G2P_UPDATE);
            return check_launch(c);
        }
        bool staged = false;
        if constexpr (sizeof(R) == 4 && OX == 1 && OY == 1 && OZ == 1) {
            if (c->tma_update && c->tune.update_ctas_per_sm == 0) {
                k_g2p_update_brick<<<c->g.nbricks, 256, 0, c->stream>>>(a);
                staged = true;
            } else if (c->tma_update) {
                const int nchunks = (int)((c->num + UCH - 1) / UCH);
                static bool attr = false;
                if (!attr) {
                    cudaFuncSetAttribute(k_g2p_update_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(2 * USTAGE));
                    cudaFuncSetAttribute(k_g2p_update_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(2 * USTAGE));
                    attr = true;
                }
                int dev = 0, nsm = 148;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
                const int grid = std::min(nchunks, nsm * c->tune.update_ctas_per_sm);
                if (c->fluid_j) launch(c->pdl != 0, k_g2p_update_tma<true>, grid, UCH, 2 * USTAGE, c->stream, a, nchunks);
                else launch(c->pdl != 0, k_g2p_update_tma<false>, grid, UCH, 2 * USTAGE, c->stream, a, nchunks);
                staged = true;
            }
        }
        if (!staged) {
            const int nb = (int)((c->num + 255) / 256);
            k_g2p_update<R, OX, OY, OZ><<<nb, 256, 0, c->stream>>>(a);
        }
        timer_end(c, K_G2P_UPDATE);
    }
    c->launches++;
    return check_launch(c);
}

template <typename R>
static mpm_status dispatch_orders(mpm_ctx *c, int which) {
    const int *o = c->g.order;
    if (o[0] == 1 && o[1] == 1 && o[2] == 1) return launch_particle_kernel<R, 1, 1, 1>(c, which);
    if (o[0] == 2 && o[1] == 2 && o[2] == 2) return launch_particle_kernel<R, 2, 2, 2>(c, which);
    if (o[0] == 2 && o[1] == 1 && o[2] == 2) return launch_particle_kernel<R, 2, 1, 2>(c, which);
    return MPM_ERR_UNSUPPORTED;
}

static mpm_status particle_kernel(mpm_ctx *c, int which) {
    return c->precision == 64 ? dispatch_orders<double>(c, which) : dispatch_orders<float>(c, which);
}

template <typename R>
static mpm_status grid_kernel(mpm_ctx *c, int which) {
    StepArgs<R> a = make_args<R>(c);
    const bool list = !a.all_tiles;
    // persistent grids of as many CTAs as reside per SM: 4 for the first pass
    // (64 registers with its batched loads), 6 for the second (40)
    const int lgrid1 = std::min(c->g.ntiles, 4 * num_sms()), lgrid = std::min(c->g.ntiles, 6 * num_sms());
    if (which == 0) {
        timer_begin(c, K_GRID1);
        if (list) {
            launch(c->pdl != 0, k_tile_list, 1, 1024, 0, c->stream, (const unsigned char *)c->d_tileflag, c->g.ntiles,
                   c->d_tlist, c->d_ntlist);
            launch(c->pdl != 0, k_grid1<R, true>, lgrid1, GRID_THREADS, 0, c->stream, a);
            c->launches++;
        } else {
            k_grid1<R, false><<<c->g.ntiles, GRID_THREADS, 0, c->stream>>>(a);
        }
        timer_end(c, K_GRID1);
    } else {
        timer_begin(c, K_GRID2);
        if (list) launch(c->pdl != 0, k_grid2<R, true>, lgrid, GRID_THREADS, 0, c->stream, a);
        else k_grid2<R, false><<<c->g.ntiles, GRID_THREADS, 0, c->stream>>>(a);
        timer_end(c, K_GRID2);
    }
    c->launches++;
    return check_launch(c);
}

mpm_status run_p2g(mpm_ctx *c, double facl) {
    c->facl = facl;
    return particle_kernel(c, 0);
}

mpm_status run_grid1(mpm_ctx *c, int) {
    return c->precision == 64 ? grid_kernel<double>(c, 0) : grid_kernel<float>(c, 0);
}

mpm_status run_g2p(mpm_ctx *c) {
    mpm_status s = particle_kernel(c, 1);
    if (s != MPM_OK) return s;
    s = c->precision == 64 ? grid_kernel<double>(c, 1) : grid_kernel<float>(c, 1);
    if (s != MPM_OK) return s;
    return particle_kernel(c, 2);
}

// ------------------------------------------------- nodal reference volume
// MakNodalVol (module/mesh.cpp:160-202), evaluated per node: the node sums
// the Gaussian-point weights of its adjacent cells.
template <int O>
__device__ __forceinline__ void axis_d(double x, double xmin, double dx, int ie, int nnc, double *w) {
    if (O == 1) {
        Axis<double, 1> a;
        axis_linear<double>(x, xmin, dx, 1.0 / dx, ie, a);
        w[0] = a.w[0]; w[1] = a.w[1];
    } else {
        Axis<double, 2> a;
        axis_quadratic<double>(x, xmin, dx, 1.0 / dx, ie, nnc, a);
        w[0] = a.w[0]; w[1] = a.w[1]; w[2] = a.w[2];
    }
}

__global__ void k_nodal_volume(Geom g, int npx, int npy, int npz, double *nvol) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.nodec) return;
    int i = n % g.nnc[0], j = (n / g.nnc[0]) % g.nnc[1], k = n / (g.nnc[0] * g.nnc[1]);
    int np[3] = {npx, npy, npz};
    int idx[3] = {i, j, k};
    double volp = g.dx[0] * g.dx[1] * g.dx[2] / (double)(npx * npy * npz);
    double wsum[3];
    for (int d = 0; d < 3; d++) {
        double s = 0.0;
        int O = g.order[d];
        for (int e = idx[d] - O; e <= idx[d]; e++) {
            if (e < 0 || e >= g.nel[d]) continue;
            for (int q = 0; q < np[d]; q++) {
                double off;
                switch (np[d]) {
                case 1: off = 0.0; break;
                case 2: off = (q == 0 ? -0.25 : 0.25); break;
                case 3: off = (q == 0 ? -1.0 / 3.0 : q == 1 ? 0.0 : 1.0 / 3.0); break;
                case 4: off = -0.375 + 0.25 * q; break;
                case 5: off = -0.4 + 0.2 * q; break;
                default: off = (-5.0 + 2.0 * q) / 12.0; break;
                }
                double xp = g.xmin[d] + g.dx[d] * (e + 0.5) + off * g.dx[d];
                double w[3];
                if (O == 1) axis_d<1>(xp, g.xmin[d], g.dx[d], e, g.nnc[d], w);
                else axis_d<2>(xp, g.xmin[d], g.dx[d], e, g.nnc[d], w);
                s += w[idx[d] - e];
            }
        }
        wsum[d] = s;
    }
    nvol[n] = wsum[0] * wsum[1] * wsum[2] * volp;
}

void launch_nodal_volume(const Geom &g, const int *npxye, double *nvol, cudaStream_t st) {
    const int nb = (g.nodec + 255) / 256;
    k_nodal_volume<<<nb, 256, 0, st>>>(g, npxye[0], npxye[1], npxye[2], nvol);
}

mpm_status compute_nodal_volume(mpm_ctx *c) {
    launch_nodal_volume(c->g, c->npxye, c->d_nvol, c->stream);
    c->launches++;
    return MPM_OK;
}

}  // namespace mpm
