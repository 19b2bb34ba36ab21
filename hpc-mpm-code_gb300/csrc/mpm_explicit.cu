// Explicit MPM transfer kernels: P2G scatter, grid update, G2P gather with
// the MUSL re-projection, and the position / deformation / stress update.
//
// One explicit step (the sequence of work/src_solid/explicit/main.cpp:39-73):
//   k_p2g         Particle2NodeS scatter  (var_trans_solid_explicit.cpp:35-70)
//   k_grid1       nvel = p/m + BC, SolveSolid a = f/m + BC, PIC v* = v + dt a,
//                 shifting nei and sum nei^2       (..:77-96, solve_solid_explicit.cpp:8-31,
//                 var_trans_solid_explicit.cpp:194-200, material_point.cpp:179-185)
//   k_g2p_musl    particle velocity gather, MUSL momentum re-scatter, |geup|^2
//                 (var_trans_solid_explicit.cpp:211-240,101-129, material_point.cpp:192-217)
//   k_grid2       MUSL nvel = p/m + BC, clears the accumulators (..:131-146)
//   k_g2p_update  F update, position update + shift, vol = J vol0, stress
//                 (..:247-296,150-185)
#include <cstdio>

#include "mpm_device.cuh"

namespace mpm {

template <typename R>
struct StepArgs {
    KGeom<R> g;
    Particles<R> P;
    const WorkItem *work;
    const int *nwork;
    unsigned long long *acc;    // NACC * nodec
    unsigned long long *acc2;   // 3 * nodec
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
    R dt, facl, mtol, grav[3];
    int parity;
    int scheme;
    int shifting;
    int all_tiles;              // process every tile in the grid passes (download mode)
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

// Scales shared by the P2G kernel (producer) and the first grid pass (consumer).
template <typename R>
struct P2GScales {
    Fix m, v, p, f;
};

template <typename R>
__device__ __forceinline__ P2GScales<R> p2g_scales(const StepArgs<R> &a) {
    const unsigned *nb = a.ctl->nxt[a.parity];
    P2GScales<R> s;
    double gabs = fmax(fabs((double)a.grav[0]), fmax(fabs((double)a.grav[1]), fabs((double)a.grav[2])));
    s.m = make_fix(a.nump * a.mmax);
    s.v = make_fix(a.nump * (double)bits_f(nb[B_VOLMAX]));
    s.p = make_fix(a.nump * a.mmax * (double)bits_f(nb[B_VMAX]));
    s.f = make_fix(a.nump * ((double)bits_f(nb[B_VOLSMAX]) * 3.0 * a.gshape + a.mmax * gabs * fabs((double)a.facl)));
    return s;
}

template <typename R>
__device__ __forceinline__ Fix musl_scale(const StepArgs<R> &a) {
    double vb = (double)bits_f(a.ctl->cur[C_GMAX]);
    if (a.scheme == MPM_FLIP) vb = (double)bits_f(a.ctl->nxt[a.parity][B_VMAX]) + fabs((double)a.dt) * vb;
    return make_fix(a.nump * a.mmax * vb * 1.0000001);
}

template <typename R>
__device__ __forceinline__ Fix geup_scale(const StepArgs<R> &a) {
    double gb = 2.0 * (double)bits_f(a.ctl->nxt[a.parity][B_VOLMAX]) * a.gsum * (double)bits_f(a.ctl->cur[C_NEIMAX]);
    return make_fix(a.nump * 3.0 * gb * gb * 1.0000001);
}

// Block-wide reductions over 256 threads (fixed order: deterministic).
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
    return r;  // valid in thread 0
}

struct OpAddD { __device__ double operator()(double a, double b) const { return a + b; } };
struct OpAddL { __device__ long long operator()(long long a, long long b) const { return a + b; } };
struct OpAddI { __device__ int operator()(int a, int b) const { return a + b; } };
struct OpMaxF { __device__ float operator()(float a, float b) const { return fmaxf(a, b); } };

// -------------------------------------------------------------------- P2G
template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(256) k_p2g(StepArgs<R> a) {
    constexpr int BX = TILE + OX, BY = TILE + OY, BZ = TILE + OZ, BOX = BX * BY * BZ;
    extern __shared__ unsigned long long sacc[];   // NACC * BOX
    __shared__ int sh_red[32];
    if ((int)blockIdx.x >= *a.nwork) return;
    const WorkItem w = a.work[blockIdx.x];
    int tx, ty, tz;
    tile_coords(w.tile, a.g.ntile, tx, ty, tz);
    const int ox = tx * TILE, oy = ty * TILE, oz = tz * TILE;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // per-step resets for the passes that follow
        for (int k = 0; k < B_NB; k++) a.ctl->nxt[a.parity ^ 1][k] = 0u;
        for (int k = 0; k < C_NC; k++) a.ctl->cur[k] = 0u;
        a.ctl->geup_acc = 0ull;
    }
    for (int i = threadIdx.x; i < NACC * BOX; i += blockDim.x) sacc[i] = 0ull;
    __syncthreads();
    const P2GScales<R> S = p2g_scales(a);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ctl->p2g_inv[0] = S.m.inv;
        a.ctl->p2g_inv[1] = S.v.inv;
        a.ctl->p2g_inv[2] = S.p.inv;
        a.ctl->p2g_inv[3] = S.f.inv;
    }
    const R fxg = a.grav[0] * a.facl, fyg = a.grav[1] * a.facl, fzg = a.grav[2] * a.facl;
    const Particles<R> &P = a.P;
    int misses = 0, oobs = 0;
    for (int p = w.begin + threadIdx.x; p < w.end; p += blockDim.x) {
        R x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        int cx = cell_of(x0, a.g, 0, oob), cy = cell_of(x1, a.g, 1, oob), cz = cell_of(x2, a.g, 2, oob);
        oobs += oob;
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        axis_eval<R, OX>(x0, a.g, 0, cx, ax);
        axis_eval<R, OY>(x1, a.g, 1, cy, ay);
        axis_eval<R, OZ>(x2, a.g, 2, cz, az);
        const R m = ld(P.m + p), vol = ld(P.vol + p);
        const R v0 = ld(P.v[0] + p), v1 = ld(P.v[1] + p), v2 = ld(P.v[2] + p);
        const R s0 = ld(P.s[0] + p), s1 = ld(P.s[1] + p), s2 = ld(P.s[2] + p);
        const R s3 = ld(P.s[3] + p), s4 = ld(P.s[4] + p), s5 = ld(P.s[5] + p);
        const R mfx = m * fxg, mfy = m * fyg, mfz = m * fzg;
        const int lx = cx - ox, ly = cy - oy, lz = cz - oz;
        const bool in = (unsigned)lx < (unsigned)TILE && (unsigned)ly < (unsigned)TILE && (unsigned)lz < (unsigned)TILE;
        misses += !in;
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R wxy = ax.w[i] * ay.w[j];
                    const R N = wxy * az.w[k];
                    const R d0 = ax.dw[i] * ay.w[j] * az.w[k];
                    const R d1 = ax.w[i] * ay.dw[j] * az.w[k];
                    const R d2 = wxy * az.dw[k];
                    const R Nm = N * m;
                    long long q[NACC];
                    q[0] = fx(Nm, S.m);
                    q[1] = fx(N * vol, S.v);
                    q[2] = fx(Nm * v0, S.p);
                    q[3] = fx(Nm * v1, S.p);
                    q[4] = fx(Nm * v2, S.p);
                    q[5] = fx(-vol * (s0 * d0 + s5 * d1 + s4 * d2) + N * mfx, S.f);
                    q[6] = fx(-vol * (s5 * d0 + s1 * d1 + s3 * d2) + N * mfy, S.f);
                    q[7] = fx(-vol * (s4 * d0 + s3 * d1 + s2 * d2) + N * mfz, S.f);
                    if (in) {
                        const int li = (lx + i) + BX * ((ly + j) + BY * (lz + k));
#pragma unroll
                        for (int f = 0; f < NACC; f++) atomic_add_i64(&sacc[f * BOX + li], q[f]);
                    } else {
                        const int gx = cx + i, gy = cy + j, gz = cz + k;
                        const int gn = gx + a.g.nnc[0] * (gy + a.g.nnc[1] * gz);
#pragma unroll
                        for (int f = 0; f < NACC; f++) atomic_add_i64(&a.acc[(size_t)f * a.g.nodec + gn], q[f]);
                        a.tileflag[tile_of_node(a.g, gx, gy, gz)] = 1;
                    }
                }
    }
    int tot = block_reduce(misses + (oobs << 16), OpAddI(), sh_red);
    if (threadIdx.x == 0 && tot) {
        if (tot & 0xffff) atomicAdd(&a.ctl->tile_misses, (unsigned)(tot & 0xffff));
        if (tot >> 16) atomicAdd(&a.ctl->err_oob, (unsigned)(tot >> 16));
    }
    __syncthreads();
    // flush the tile box to the global accumulators
    for (int li = threadIdx.x; li < BOX; li += blockDim.x) {
        const int lx = li % BX, ly = (li / BX) % BY, lz = li / (BX * BY);
        const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        const int gn = gx + a.g.nnc[0] * (gy + a.g.nnc[1] * gz);
        bool any = false;
#pragma unroll
        for (int f = 0; f < NACC; f++) {
            unsigned long long v = sacc[f * BOX + li];
            if (v) {
                atomicAdd(&a.acc[(size_t)f * a.g.nodec + gn], v);
                any = true;
            }
        }
        if (any) a.tileflag[tile_of_node(a.g, gx, gy, gz)] = 1;
    }
}

// ------------------------------------------------------------ grid pass 1
template <typename R>
__global__ void __launch_bounds__(256) k_grid1(StepArgs<R> a) {
    __shared__ double sh_d[32];
    __shared__ float sh_f[32];
    __shared__ bool s_last;
    const int t = blockIdx.x;
    double eu = 0.0;
    float gmax = 0.0f, neimax = 0.0f;
    if (a.all_tiles || a.tileflag[t]) {
        const P2GScales<R> S = p2g_scales(a);
        int tx, ty, tz;
        tile_coords(t, a.g.ntile, tx, ty, tz);
        const size_t N = (size_t)a.g.nodec;
        for (int li = threadIdx.x; li < TILE * TILE * TILE; li += blockDim.x) {
            const int gx = tx * TILE + (li % TILE), gy = ty * TILE + (li / TILE) % TILE, gz = tz * TILE + li / (TILE * TILE);
            if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
            const size_t n = gx + (size_t)a.g.nnc[0] * (gy + (size_t)a.g.nnc[1] * gz);
            const R mass = (R)((double)(long long)a.acc[n] * S.m.inv);
            R vof = (R)((double)(long long)a.acc[N + n] * S.v.inv);
            R nv[3], na[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const R pc = (R)((double)(long long)a.acc[(2 + c) * N + n] * S.p.inv);
                const R fc = (R)((double)(long long)a.acc[(5 + c) * N + n] * S.f.inv);
                nv[c] = (mass > a.mtol) ? pc / mass : (R)0;
                na[c] = (mass > a.mtol) ? fc / mass : (R)0;
            }
            if (vof < a.mtol) vof = (R)0;
            const unsigned char bf = a.bcflag[n];
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
            R e = vof - (R)a.nvol[n];
            e = e > (R)0 ? e : (R)0;
            a.nei[n] = e;
            eu += (double)e * (double)e;
            neimax = fmaxf(neimax, (float)e);
        }
    }
    // deterministic sum of nei^2: per-tile partials, reduced in tile order by the last CTA
    double ebl = block_reduce(eu, OpAddD(), sh_d);
    float gm = block_reduce(gmax, OpMaxF(), sh_f);
    float nm = block_reduce(neimax, OpMaxF(), sh_f);
    if (threadIdx.x == 0) {
        a.eu_part[t] = ebl;
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
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) acc += ((volatile double *)a.eu_part)[i];
        double tot = block_reduce(acc, OpAddD(), sh_d);
        if (threadIdx.x == 0) {
            a.ctl->eu_norm = tot;
            a.ctl->tile_counter = 0u;
        }
    }
}

// ------------------------------------------------------ G2P 1 + MUSL scatter
template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(256) k_g2p_musl(StepArgs<R> a) {
    constexpr int BX = TILE + OX, BY = TILE + OY, BZ = TILE + OZ, BOX = BX * BY * BZ;
    extern __shared__ unsigned long long sacc[];   // 3 * BOX
    __shared__ long long sh_l[32];
    __shared__ float sh_f[32];
    if ((int)blockIdx.x >= *a.nwork) return;
    const WorkItem w = a.work[blockIdx.x];
    int tx, ty, tz;
    tile_coords(w.tile, a.g.ntile, tx, ty, tz);
    const int ox = tx * TILE, oy = ty * TILE, oz = tz * TILE;
    for (int i = threadIdx.x; i < 3 * BOX; i += blockDim.x) sacc[i] = 0ull;
    __syncthreads();
    const Fix SQ = musl_scale(a);
    const Fix SG = geup_scale(a);
    const size_t N = (size_t)a.g.nodec;
    const Particles<R> &P = a.P;
    const bool flip = (a.scheme == MPM_FLIP);
    long long gacc = 0;
    float vmax = 0.0f;
    for (int p = w.begin + threadIdx.x; p < w.end; p += blockDim.x) {
        R x0 = ld(P.x[0] + p), x1 = ld(P.x[1] + p), x2 = ld(P.x[2] + p);
        bool oob = false;
        int cx = cell_of(x0, a.g, 0, oob), cy = cell_of(x1, a.g, 1, oob), cz = cell_of(x2, a.g, 2, oob);
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
        // gather: PIC v = sum N v*, FLIP v += sum N dt a (PIC/FLIP::VarG2P, map_and_interpolate.h:12-55)
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R wxy = ax.w[i] * ay.w[j];
                    const R N_ = wxy * az.w[k];
                    const size_t gn = (cx + i) + (size_t)a.g.nnc[0] * ((cy + j) + (size_t)a.g.nnc[1] * (cz + k));
                    if (flip) {
                        const R Nd = N_ * a.dt;
#pragma unroll
                        for (int c = 0; c < 3; c++) v[c] += Nd * ld(a.G + c * N + gn);
                    } else {
#pragma unroll
                        for (int c = 0; c < 3; c++) v[c] += N_ * ld(a.G + c * N + gn);
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
        // |geup|^2 with geup = 2 vol sum dN nei (material_point.cpp:192-216)
        const R tv = (R)2 * vol;
        const R g0 = gu[0] * tv, g1 = gu[1] * tv, g2 = gu[2] * tv;
        gacc += fx((double)g0 * (double)g0 + (double)g1 * (double)g1 + (double)g2 * (double)g2, SG);
        // MUSL re-projection of momentum (var_trans_solid_explicit.cpp:108-129)
        const int lx = cx - ox, ly = cy - oy, lz = cz - oz;
        const bool in = (unsigned)lx < (unsigned)TILE && (unsigned)ly < (unsigned)TILE && (unsigned)lz < (unsigned)TILE;
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R Nm = ax.w[i] * ay.w[j] * az.w[k] * m;
                    long long q0 = fx(Nm * v[0], SQ), q1 = fx(Nm * v[1], SQ), q2 = fx(Nm * v[2], SQ);
                    if (in) {
                        const int li = (lx + i) + BX * ((ly + j) + BY * (lz + k));
                        atomic_add_i64(&sacc[li], q0);
                        atomic_add_i64(&sacc[BOX + li], q1);
                        atomic_add_i64(&sacc[2 * BOX + li], q2);
                    } else {
                        const size_t gn = (cx + i) + (size_t)a.g.nnc[0] * ((cy + j) + (size_t)a.g.nnc[1] * (cz + k));
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
        const size_t gn = gx + (size_t)a.g.nnc[0] * (gy + (size_t)a.g.nnc[1] * gz);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            unsigned long long v = sacc[c * BOX + li];
            if (v) atomicAdd(&a.acc2[c * N + gn], v);
        }
    }
}

// ------------------------------------------------------------ grid pass 2
template <typename R>
__global__ void __launch_bounds__(256) k_grid2(StepArgs<R> a) {
    const int t = blockIdx.x;
    if (!(a.all_tiles || a.tileflag[t])) return;
    const P2GScales<R> S = p2g_scales(a);
    const Fix SQ = musl_scale(a);
    int tx, ty, tz;
    tile_coords(t, a.g.ntile, tx, ty, tz);
    const size_t N = (size_t)a.g.nodec;
    for (int li = threadIdx.x; li < TILE * TILE * TILE; li += blockDim.x) {
        const int gx = tx * TILE + (li % TILE), gy = ty * TILE + (li / TILE) % TILE, gz = tz * TILE + li / (TILE * TILE);
        if (gx >= a.g.nnc[0] || gy >= a.g.nnc[1] || gz >= a.g.nnc[2]) continue;
        const size_t n = gx + (size_t)a.g.nnc[0] * (gy + (size_t)a.g.nnc[1] * gz);
        const R mass = (R)((double)(long long)a.acc[n] * S.m.inv);
        R nv[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const R pc = (R)((double)(long long)a.acc2[c * N + n] * SQ.inv);
            nv[c] = (mass > a.mtol) ? pc / mass : (R)0;
        }
        const unsigned char bf = a.bcflag[n];
        if (bf) {
#pragma unroll
            for (int c = 0; c < 3; c++)
                if (bf & (1 << c)) nv[c] = a.bcval[c * N + n] * a.facl;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) a.nvel2[c * N + n] = nv[c];
        if (!a.all_tiles) {
#pragma unroll
            for (int f = 0; f < NACC; f++) a.acc[f * N + n] = 0ull;
#pragma unroll
            for (int c = 0; c < 3; c++) a.acc2[c * N + n] = 0ull;
        }
    }
    if (!a.all_tiles) {
        __syncthreads();
        if (threadIdx.x == 0) a.tileflag[t] = 0;
    }
}

// ----------------------------------------------- G2P 2: F, x, vol, stress
template <typename R, int OX, int OY, int OZ>
__global__ void __launch_bounds__(256) k_g2p_update(StepArgs<R> a) {
    __shared__ float sh_f[32];
    __shared__ int sh_i[32];
    if ((int)blockIdx.x >= *a.nwork) return;
    const WorkItem w = a.work[blockIdx.x];
    const size_t N = (size_t)a.g.nodec;
    const Particles<R> &P = a.P;
    // b0 of DeltaCorrectionParticleShifting (material_point.cpp:219)
    double b0 = 0.0;
    if (a.shifting) {
        const Fix SG = geup_scale(a);
        double gd = (double)(long long)a.ctl->geup_acc * SG.inv;
        b0 = (gd < (double)a.mtol) ? 0.0 : a.ctl->eu_norm / gd;
    }
    const R rb0 = (R)b0;
    float volmax = 0.0f, vsmax = 0.0f;
    int bad = 0;
    for (int p = w.begin + threadIdx.x; p < w.end; p += blockDim.x) {
        R x[3] = {ld(P.x[0] + p), ld(P.x[1] + p), ld(P.x[2] + p)};
        bool oob = false;
        int cx = cell_of(x[0], a.g, 0, oob), cy = cell_of(x[1], a.g, 1, oob), cz = cell_of(x[2], a.g, 2, oob);
        Axis<R, OX> ax;
        Axis<R, OY> ay;
        Axis<R, OZ> az;
        axis_eval<R, OX>(x[0], a.g, 0, cx, ax);
        axis_eval<R, OY>(x[1], a.g, 1, cy, ay);
        axis_eval<R, OZ>(x[2], a.g, 2, cz, az);
        R D[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        R xn[3] = {x[0], x[1], x[2]};
        R gu[3] = {(R)0, (R)0, (R)0};
#pragma unroll
        for (int k = 0; k <= OZ; k++)
#pragma unroll
            for (int j = 0; j <= OY; j++)
#pragma unroll
                for (int i = 0; i <= OX; i++) {
                    const R wxy = ax.w[i] * ay.w[j];
                    const R N_ = wxy * az.w[k];
                    const R dn[3] = {ax.dw[i] * ay.w[j] * az.w[k], ax.w[i] * ay.dw[j] * az.w[k], wxy * az.dw[k]};
                    const size_t gn = (cx + i) + (size_t)a.g.nnc[0] * ((cy + j) + (size_t)a.g.nnc[1] * (cz + k));
                    const R nv[3] = {ld(a.nvel2 + gn), ld(a.nvel2 + N + gn), ld(a.nvel2 + 2 * N + gn)};
#pragma unroll
                    for (int r = 0; r < 3; r++)
#pragma unroll
                        for (int c = 0; c < 3; c++) D[r][c] += dn[c] * nv[r] * a.dt;
                    const R Nd = N_ * a.dt;
#pragma unroll
                    for (int c = 0; c < 3; c++) xn[c] += Nd * nv[c];   // FLIP::VarG2P on coord
                    if (rb0 != (R)0) {
                        const R e = ld(a.nei + gn);
#pragma unroll
                        for (int c = 0; c < 3; c++) gu[c] += dn[c] * e;
                    }
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
        if (sizeof(R) == 8) {
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
        } else {
            // FP32: F + D F keeps the small increment out of the rounding of I + D
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    R acc = F[r][c];
#pragma unroll
                    for (int k2 = 0; k2 < 3; k2++) acc += D[r][k2] * F[k2][c];
                    Fn[r][c] = acc;
                    Dm[r][c] = D[r][c];
                }
        }
        const R J = det3(Fn);
        const R volp = J * ld(P.vol0 + p);
        R s[6];
#pragma unroll
        for (int k = 0; k < 6; k++) s[k] = ld(P.s[k] + p);
        const int mid = P.matid[p];
        const int model = a.iprop[mid];
        const R E = (R)a.matprop[3 * mid], nu = (R)a.matprop[3 * mid + 1];
        if (model == 0) {
            lin_elast_update(s, Dm, E, nu);
        } else if (model == 1) {
            neo_hookean_stress(s, Fn, J, E, nu);
        } else if (model == -1) {
#pragma unroll
            for (int k = 0; k < 6; k++) s[k] = (R)0;
        }
        bool fin = isfinite(xn[0]) && isfinite(xn[1]) && isfinite(xn[2]) && isfinite(J) && isfinite(s[0]) &&
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
        volmax = fmaxf(volmax, vf);
        vsmax = fmaxf(vsmax, vf * fmaxf(rs0, fmaxf(rs1, rs2)));
    }
    float vm = block_reduce(volmax, OpMaxF(), sh_f);
    float sm = block_reduce(vsmax, OpMaxF(), sh_f);
    int nb = block_reduce(bad, OpAddI(), sh_i);
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
        a.grav[d] = (R)c->gravity[d];
    }
    a.g.nodec = c->g.nodec;
    char *base = (char *)c->pbuf[c->cur];
    size_t n = (size_t)c->num, rs = sizeof(R);
    R *f = (R *)base;
    for (int k = 0; k < 3; k++) a.P.x[k] = f + (0 + k) * n;
    for (int k = 0; k < 3; k++) a.P.v[k] = f + (3 + k) * n;
    for (int k = 0; k < 9; k++) a.P.F[k] = f + (6 + k) * n;
    for (int k = 0; k < 6; k++) a.P.s[k] = f + (15 + k) * n;
    a.P.m = f + 21 * n;
    a.P.vol0 = f + 22 * n;
    a.P.vol = f + 23 * n;
    a.P.matid = (int *)(base + 24 * n * rs);
    a.P.pid = a.P.matid + n;
    a.work = c->d_work;
    a.nwork = c->d_nwork;
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
    a.dt = (R)c->dt;
    a.facl = (R)c->facl;
    a.mtol = (R)c->mtol;
    a.parity = (int)(c->step & 1);
    a.scheme = c->scheme;
    a.shifting = c->shifting;
    a.all_tiles = c->write_nodal_dl ? 1 : 0;
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

template <typename R, int OX, int OY, int OZ>
static mpm_status launch_particle_kernel(mpm_ctx *c, int which) {
    StepArgs<R> a = make_args<R>(c);
    constexpr int BOX = (TILE + OX) * (TILE + OY) * (TILE + OZ);
    const int grid = c->nwork_cap;
    if (grid == 0) return MPM_OK;
    if (which == 0) {
        size_t smem = (size_t)NACC * BOX * sizeof(unsigned long long);
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(k_p2g<R, OX, OY, OZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            attr = true;
        }
        timer_begin(c, K_P2G);
        k_p2g<R, OX, OY, OZ><<<grid, 256, smem, c->stream>>>(a);
        timer_end(c, K_P2G);
    } else if (which == 1) {
        size_t smem = (size_t)3 * BOX * sizeof(unsigned long long);
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(k_g2p_musl<R, OX, OY, OZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            attr = true;
        }
        timer_begin(c, K_G2P_MUSL);
        k_g2p_musl<R, OX, OY, OZ><<<grid, 256, smem, c->stream>>>(a);
        timer_end(c, K_G2P_MUSL);
    } else {
        timer_begin(c, K_G2P_UPDATE);
        k_g2p_update<R, OX, OY, OZ><<<grid, 256, 0, c->stream>>>(a);
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
    if (which == 0) {
        timer_begin(c, K_GRID1);
        k_grid1<R><<<c->g.ntiles, 256, 0, c->stream>>>(a);
        timer_end(c, K_GRID1);
    } else {
        timer_begin(c, K_GRID2);
        k_grid2<R><<<c->g.ntiles, 256, 0, c->stream>>>(a);
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
    // per direction: sum over adjacent cells e (ie - order .. ie) of the weights at the Gaussian points
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

mpm_status compute_nodal_volume(mpm_ctx *c) {
    int nb = (c->g.nodec + 255) / 256;
    k_nodal_volume<<<nb, 256, 0, c->stream>>>(c->g, c->npxye[0], c->npxye[1], c->npxye[2], c->d_nvol);
    c->launches++;
    return MPM_OK;
}

}  // namespace mpm
