// Internal declarations of the GB300 MPM transfer path.
//
// Data layout in HBM
//   particles: structure of arrays, one array per scalar component, in the
//     context's precision R (float or double): x[3], v[3], F[9] (row major;
//     FP32 stores the displacement gradient F - I in these arrays), each
//     array pstride (num rounded up to 64) elements long so that every
//     array starts 256-byte aligned for bulk asynchronous copies,
//     sigma[6] (Voigt xx,yy,zz,yz,xz,xy), m, vol0, vol; plus matid and the
//     particle's load index (pid).  Two copies exist; a re-sort permutes A
//     into B and swaps.
//   grid: node n = i + nx*(j + ny*k) exactly as MakSf numbers control points
//     (module/shape_function.cpp:28); vector fields component-major.
//     P2G sums are int64 fixed point, field-major: acc[f*nodec + n].
//   tiles: 8x8x8 blocks of cells/nodes.  Particles are kept grouped by the
//     tile of their cell; a "work item" is a chunk of one tile's particles
//     and is the unit one CTA processes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "mpm_gpu.h"

namespace mpm {

constexpr int TILE = 8;              // node tile edge for the grid passes and activity flags
constexpr int BRX = 4, BRY = 4, BRZ = 8;   // particle brick: cells per brick edge
constexpr int BRC = BRX * BRY * BRZ;       // cells per brick (one CTA thread per cell)
constexpr int CHUNK = 1024;          // max particles per work item
constexpr int SCAN_SEG = 4096;       // bricks per segment of the brick-count scan (mpm_sort.cu)
constexpr int NACC = 8;              // P2G fields: mass, vof, mome xyz, force xyz
constexpr int NKCLASS = 14;          // kernel classes for timing

enum KernelClass {
    K_BIN = 0, K_SCAN, K_SCATTER, K_PERMUTE, K_P2G, K_GRID1, K_G2P_MUSL, K_GRID2, K_G2P_UPDATE, K_MISC,
    K_MATVEC, K_KRYLOV, K_ASSEMBLE, K_PRECOND
};

struct Geom {
    int nel[3];      // cells
    int nnc[3];      // control points per direction (nel + order)
    int order[3];    // 1 or 2
    int ntile[3];    // node tiles per direction (over control points)
    int ntiles;
    int nbrick[3];   // particle bricks per direction (over cells)
    int nbricks;
    int nodec;
    int nelem;
    double xmin[3], dx[3];
};

// Bounds that set the fixed-point scales.  Values are non-negative floats
// stored as their bit patterns so that atomicMax on unsigned int orders them.
enum BoundSlot { B_VMAX = 0, B_VOLMAX, B_VOLSMAX, B_AMAX, B_NB };   // produced for the next step
enum CurSlot { C_GMAX = 0, C_NEIMAX, C_JVMAX, C_NC };                    // produced and used within a step

// Fixed-point scale 2^e, applied as two float factors so that e up to +-250
// never overflows an intermediate.
struct Fix {
    float s1, s2;   // s1 * s2 = 2^e
    float i1, i2;   // i1 * i2 = 2^-e
    double sd;      // 2^e
    double inv;     // 2^-e
};

// Fixed-point scales of one step (see make_fix).
struct Scales {
    Fix m, v, p, f;   // P2G: mass, vof, momentum, force
    Fix q;            // MUSL momentum
    Fix gd;           // |geup|^2
};

struct DevCtl {
    unsigned int nxt[2][B_NB];
    unsigned int cur[C_NC];
    unsigned long long geup_acc;     // fixed-point sum of |geup|^2
    double eu_norm;                  // sum nei^2 (deterministic per-tile reduction)
    unsigned int tile_counter;
    unsigned int err_oob;
    unsigned int err_nonfinite;
    unsigned int tile_misses;
    double p2g_inv[4];               // 2^-e of the P2G scales (mass, vof, momentum, force) of the last P2G
    double b0;                       // shifting coefficient of this step
    unsigned int err_timeout;        // bounded device waits that gave up
    unsigned int n_miss_p2g;         // particles queued for the deferred P2G pass this step
    unsigned int n_miss_musl;        // particles queued for the deferred gather/MUSL pass this step
    Scales sc_p2g;                   // this step's P2G scales (k_step_reset)
    Scales sc_musl;                  // this step's gather/MUSL scales (last CTA of k_grid1)
    Fix sc_fbar;                     // F-bar: scale of the projected J vol sums (k_fbar_scale)
};

template <typename R>
struct Particles {
    R *x[3], *v[3], *F[9], *s[6], *m, *vol0, *vol;
    R *a[3];          // particle acceleration (implicit contexts only, else null)
    R *C[9];          // affine velocity matrix, row major (TPIC / APIC contexts only, else null)
    R *Fb[9], *Jb, *Jt;   // F-bar contexts: def_grad_bar, det_def_grad_bar, trial J of the step (FP32: all minus I / 1)
    int *matid, *pid;
};

struct WorkItem {
    int tile;
    int begin;
    int end;
};


// Launch variants.  The ones mpm_gpu_autotune chooses between from measured
// times (staged or direct, resident CTAs per SM) give bitwise identical
// results; the moment forms (the defaults) differ from the corner forms by
// FP32 rounding only and are not switched by the autotuner.
struct Tune {
    int p2g_moments = 1;            // FP32 P2G in moment form (k_p2g_cell_mom); 0: corner sums
    int brick_list = 1;             // moment P2G and gather + MUSL walk the list of bricks holding particles
    int p2g_staged = 0;             // per-cell P2G reads the brick's particles from bulk-copied shared memory
    int p2g_minb = 2;               // resident CTAs the direct per-cell P2G is compiled for (2 or 3)
    int musl_staged = 0;            // gather + MUSL reads the brick's particles from staged shared memory
    int musl_minb = 3;              // resident CTAs the direct gather + MUSL kernel is compiled for
    int musl_moments = 2;           // FP32 gather + MUSL in moment form (k_g2p_musl_mom, 1: 3 / 2: 2 resident CTAs per SM); 0: corner form
    int update_ctas_per_sm = 3;     // persistent CTAs per SM of the staged particle update (0: per-brick update)
    bool done = false;
};

// two tunings that launch the same kernels (a captured graph stays valid)
inline bool same_launches(const Tune &x, const Tune &y) {
    return x.p2g_moments == y.p2g_moments && x.brick_list == y.brick_list && x.p2g_staged == y.p2g_staged &&
           x.p2g_minb == y.p2g_minb && x.musl_staged == y.musl_staged && x.musl_minb == y.musl_minb &&
           x.musl_moments == y.musl_moments && x.update_ctas_per_sm == y.update_ctas_per_sm;
}

struct KernelTimer {
    bool on = false;
    std::vector<cudaEvent_t> ev;      // pairs
    std::vector<int> cls;
    double ms[NKCLASS] = {0};
    int64_t launches[NKCLASS] = {0};
};

}  // namespace mpm

struct mpm_ctx {
    mpm::Geom g;
    int precision = 32;
    int scheme = 0;
    int shifting = 1;
    int resort_period = 8;
    double dt = 0, mtol = 0, gravity[3] = {0, 0, 0};
    double facl = 1.0;
    int nmat = 0;
    bool sigma_in = false;   // a material updates its stress incrementally (model 0 reads sigma)
    int npxye[3] = {1, 1, 1};
    cudaStream_t stream = nullptr;
    // host I/O pipeline of mpm_gpu_steps_host: copy streams and per-field events
    cudaStream_t io_h2d = nullptr, io_d2h = nullptr;
    static constexpr int IO_MAX_CHUNKS = 16;
    int io_chunks = 4;   // pieces per field copy in the host I/O pipeline (env MPM_GB300_IO_CHUNKS)
    // [0, 5 M) uploads done, [5 M, 10 M) downloads done, then gather done, start (M = IO_MAX_CHUNKS)
    cudaEvent_t io_ev[10 * IO_MAX_CHUNKS + 2] = {};
    // materials on device
    int *d_iprop = nullptr;
    double *d_matprop = nullptr;
    float *d_matpropf = nullptr;   // FP32 copy of the material table for the FP32 particle kernels
    // particles
    int64_t num = 0;
    size_t rsize = 4;
    int nreal = 24;                        // real fields per particle: 24, 27 with acceleration (implicit),
                                           // 33 with the affine matrix (TPIC / APIC)
    bool affine = false;                   // TPIC or APIC: fields [24, 33) hold the affine matrix
    bool fbar = false;                     // F-bar: 11 fields from off_fbar (Fbar 9, Jbar, trial J)
    bool fluid_j = false;                  // FP32, every material a Tait fluid: field 6 holds J - 1 and the other
                                           // eight deformation-gradient fields are neither read nor written
    int off_fbar = 0;
    size_t pstride = 64;                   // elements between particle field arrays: num rounded up to 64
    void *pbuf[2] = {nullptr, nullptr};   // two SoA copies
    int cur = 0;
    double mmax = 0.0;
    // grid
    unsigned long long *d_acc = nullptr;   // NACC * nodec int64 P2G sums
    unsigned long long *d_acc2 = nullptr;  // 3 * nodec int64 MUSL momentum
    unsigned long long *d_facc = nullptr;  // nodec int64 F-bar sums of N J vol (F-bar contexts)
    void *d_nodal = nullptr;               // R: gather field G (3), nei (1), nvel2 (3), nvel (3), naccel (3)
    double *d_nvol = nullptr;              // nodal reference volume (FP64)
    unsigned char *d_bcflag = nullptr;     // bit c: component c constrained
    void *d_bcval = nullptr;               // R[3*nodec] prescribed values
    unsigned char *d_tileflag = nullptr;
    double *d_eu_part = nullptr;
    // sorting
    int *d_key = nullptr, *d_perm = nullptr, *d_tcount = nullptr, *d_tstart = nullptr, *d_tcursor = nullptr;
    int *d_tmp = nullptr, *d_perm2 = nullptr;   // per-brick cell sort
    int *d_cstart = nullptr;                    // nbricks * (BRC + 1) cell start offsets
    int *d_scanpart = nullptr;                  // per-segment sums of the brick-count scan (3 per segment + totals)
    double *d_stage = nullptr;                  // FP64 AoS staging for host <-> device particle state
    mpm::WorkItem *d_work = nullptr;
    int *d_nwork = nullptr;
    int *d_blist = nullptr;       // bricks holding particles, in brick order (rebuilt by every sort)
    int *d_nblist = nullptr;
    int *d_tlist = nullptr;       // active node tiles of the current step (tile order)
    int *d_ntlist = nullptr;
    int nwork_cap = 0;
    int nwork = 0;
    mpm::DevCtl *d_ctl = nullptr;
    mpm::DevCtl *h_ctl = nullptr;          // pinned mirror
    // state
    int64_t step = 0;
    int64_t resorts = 0;
    int64_t launches = 0;
    int64_t steps_since_sort = 1 << 30;
    int stage = 0;   // 0 idle, 1 after p2g, 2 after grid update
    bool accum_dirty = false;
    bool write_nodal_dl = false;
    int cell_scatter = 1;   // FP32 linear: per-cell register scatter (else staging-box atomics)
    int tma_update = 1;     // FP32 linear: particle update with bulk-copy staged input
    int pdl = 1;            // step kernels launched with programmatic dependent launch (MPM_GB300_PDL=0: off)
    int alternate = 1;      // particle kernels walk bricks / chunks in alternating directions (MPM_GB300_ALTERNATE=0: forward)
    mpm_status latched = MPM_OK;
    mpm::KernelTimer timer;
    mpm::Tune tune;
    // CUDA graph of 2 x resort_period fused explicit steps (mpm_gpu_step_explicit)
    int use_graph = 1;
    int gather_norm = 1;   // FP32 gathers divide by their weight sum (MPM_GB300_GATHER_NORM=0: off)
    cudaGraphExec_t graph_exec = nullptr;
    double graph_facl = 0.0;
    cudaStream_t graph_stream = nullptr;
    mpm::Tune graph_tune;
    int graph_cur = 0;
    void *graph_pbuf[2] = {nullptr, nullptr};
    int64_t graph_launches = 0;
    int64_t graph_replays = 0;
    struct ImpState *imp = nullptr;   // implicit solid state (mpm_implicit.cu)
    std::vector<int> bc_nodes[3];
    std::vector<double> bc_vals[3];
};

namespace mpm {
// mpm_sort.cu
mpm_status sort_particles(mpm_ctx *c);
// mpm_implicit.cu
void implicit_free(mpm_ctx *c);
mpm_status implicit_bc_changed(mpm_ctx *c);   // after mpm_gpu_set_bc on an implicit context
// mpm_explicit.cu
mpm_status run_p2g(mpm_ctx *c, double facl);
mpm_status run_grid1(mpm_ctx *c, int mode);
mpm_status run_g2p(mpm_ctx *c);
mpm_status compute_nodal_volume(mpm_ctx *c);
// MakNodalVol (module/mesh.cpp:160-202) of grid g into nvol (nodec) on st
void launch_nodal_volume(const Geom &g, const int *npxye, double *nvol, cudaStream_t st);
// timing helpers (mpm_ctx.cu)
void timer_begin(mpm_ctx *c, int cls);
void timer_end(mpm_ctx *c, int cls);
mpm_status check_launch(mpm_ctx *c);
}  // namespace mpm
