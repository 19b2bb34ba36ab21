// C ABI of the GB300 MPM transfer path: context lifetime, particle load,
// boundary conditions, the explicit step and result downloads.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "mpm_device.cuh"

using namespace mpm;

namespace mpm {

static const char *kClassNames[NKCLASS] = {"bin",  "scan", "scatter", "permute", "p2g",    "grid1",
                                           "g2p_musl", "grid2", "g2p_update", "misc", "matvec", "krylov",
                                           "assemble", "precond_nn"};

void timer_begin(mpm_ctx *c, int cls) {
    if (!c->timer.on) return;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c->stream);
    c->timer.ev.push_back(e0);
    c->timer.ev.push_back(e1);
    c->timer.cls.push_back(cls);
}

void timer_end(mpm_ctx *c, int) {
    if (!c->timer.on) return;
    cudaEventRecord(c->timer.ev.back(), c->stream);
}

mpm_status check_launch(mpm_ctx *c) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "mpm_gb300: CUDA error %s\n", cudaGetErrorString(e));
        c->latched = MPM_ERR_CUDA;
        return MPM_ERR_CUDA;
    }
    return MPM_OK;
}

}  // namespace mpm

#define CK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t _e = (call);                                                                                       \
        if (_e != cudaSuccess) {                                                                                       \
            fprintf(stderr, "mpm_gb300: %s failed: %s\n", #call, cudaGetErrorString(_e));                              \
            return _e == cudaErrorMemoryAllocation ? MPM_ERR_OOM : MPM_ERR_CUDA;                                       \
        }                                                                                                              \
    } while (0)

void drop_graph(mpm_ctx *c);

static void free_dev(void *p) {
    if (p) cudaFree(p);
}

static void free_particles(mpm_ctx *c) {
    free_dev(c->pbuf[0]);
    free_dev(c->pbuf[1]);
    free_dev(c->d_key);
    free_dev(c->d_perm);
    free_dev(c->d_tmp);
    free_dev(c->d_perm2);
    free_dev(c->d_stage);
    free_dev(c->d_work);
    c->pbuf[0] = c->pbuf[1] = nullptr;
    c->d_key = c->d_perm = c->d_tmp = c->d_perm2 = nullptr;
    c->d_stage = nullptr;
    c->d_work = nullptr;
    c->num = 0;
}

// The exported functions take C linkage from their declarations in mpm_gpu.h.

const char *mpm_gpu_status_string(mpm_status s) {
    switch (s) {
    case MPM_OK: return "ok";
    case MPM_ERR_BAD_ARG: return "bad argument";
    case MPM_ERR_OOM: return "out of device memory";
    case MPM_ERR_NONFINITE: return "non-finite particle state";
    case MPM_ERR_PARTICLE_OUT_OF_BOX: return "particle outside the grid";
    case MPM_ERR_KRYLOV_MAXIT: return "Krylov solver reached its iteration limit";
    case MPM_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case MPM_ERR_CUDA: return "CUDA error";
    case MPM_ERR_STATE: return "call out of order";
    case MPM_ERR_UNSUPPORTED: return "unsupported configuration";
    case MPM_ERR_NEWTON_MAXIT: return "Newton iteration did not converge";
    }
    return "unknown";
}

mpm_status mpm_gpu_create(const mpm_grid_desc *grid, const mpm_material_desc *mat, const mpm_config *cfg,
                          mpm_ctx **out) {
    if (!grid || !mat || !cfg || !out) return MPM_ERR_BAD_ARG;
    *out = nullptr;
    if (cfg->precision != 32 && cfg->precision != 64) return MPM_ERR_BAD_ARG;
    if (cfg->scheme < MPM_PIC || cfg->scheme > MPM_APIC) return MPM_ERR_UNSUPPORTED;
    if (cfg->implicit && cfg->scheme > MPM_FLIP) return MPM_ERR_UNSUPPORTED;
    if (cfg->implicit && cfg->fbar) return MPM_ERR_UNSUPPORTED;
    if (!(cfg->dt > 0.0) || mat->nmat <= 0 || !mat->iprop || !mat->mat_prop) return MPM_ERR_BAD_ARG;
    for (int d = 0; d < 3; d++) {
        if (grid->xyelem[d] <= 0 || !(grid->dxy[d] > 0.0)) return MPM_ERR_BAD_ARG;
        if (grid->idimc[d] != 1 && grid->idimc[d] != 2) return MPM_ERR_UNSUPPORTED;
        if (grid->npxye[d] < 1 || grid->npxye[d] > 6) return MPM_ERR_BAD_ARG;
    }
    {
        const int *o = grid->idimc;
        bool ok = (o[0] == 1 && o[1] == 1 && o[2] == 1) || (o[0] == 2 && o[1] == 2 && o[2] == 2) ||
                  (o[0] == 2 && o[1] == 1 && o[2] == 2);
        if (!ok) return MPM_ERR_UNSUPPORTED;
    }
    for (int k = 0; k < mat->nmat; k++)
        if (mat->iprop[k] < -1 || mat->iprop[k] > 4) return MPM_ERR_UNSUPPORTED;
    mpm_ctx *c = new (std::nothrow) mpm_ctx();
    if (!c) return MPM_ERR_OOM;
    if (const char *gn = getenv("MPM_GB300_GATHER_NORM")) c->gather_norm = atoi(gn) != 0;
    if (const char *al = getenv("MPM_GB300_ALTERNATE")) c->alternate = atoi(al) != 0;
    if (const char *pd = getenv("MPM_GB300_PDL")) c->pdl = atoi(pd) != 0;
    if (const char *ic = getenv("MPM_GB300_IO_CHUNKS"))
        c->io_chunks = std::max(1, std::min(mpm_ctx::IO_MAX_CHUNKS, atoi(ic)));
    Geom &g = c->g;
    long long nodec = 1;
    for (int d = 0; d < 3; d++) {
        g.nel[d] = grid->xyelem[d];
        g.order[d] = grid->idimc[d];
        g.nnc[d] = grid->xyelem[d] + grid->idimc[d];
        g.ntile[d] = (g.nnc[d] + TILE - 1) / TILE;
        g.xmin[d] = grid->xymin[d];
        g.dx[d] = grid->dxy[d];
        c->npxye[d] = grid->npxye[d];
        c->gravity[d] = cfg->gravity[d];
        nodec *= g.nnc[d];
    }
    if (nodec > (1LL << 30)) {
        delete c;
        return MPM_ERR_BAD_ARG;
    }
    g.nodec = (int)nodec;
    g.nelem = g.nel[0] * g.nel[1] * g.nel[2];
    g.ntiles = g.ntile[0] * g.ntile[1] * g.ntile[2];
    g.nbrick[0] = (g.nel[0] + BRX - 1) / BRX;
    g.nbrick[1] = (g.nel[1] + BRY - 1) / BRY;
    g.nbrick[2] = (g.nel[2] + BRZ - 1) / BRZ;
    g.nbricks = g.nbrick[0] * g.nbrick[1] * g.nbrick[2];
    c->precision = cfg->precision;
    c->rsize = cfg->precision == 64 ? 8 : 4;
    c->scheme = cfg->scheme;
    c->shifting = cfg->shifting ? 1 : 0;
    c->resort_period = cfg->resort_period > 0 ? cfg->resort_period : 8;
    c->cell_scatter = cfg->scatter == 1 ? 0 : 1;
    c->affine = cfg->scheme == MPM_TPIC || cfg->scheme == MPM_APIC;
    c->fbar = cfg->fbar != 0;
    c->off_fbar = c->affine ? 33 : 24;
    c->nreal = cfg->implicit ? 27 : c->off_fbar + (c->fbar ? 11 : 0);
    c->dt = cfg->dt;
    c->mtol = cfg->mtol;
    c->nmat = mat->nmat;
    size_t N = (size_t)g.nodec;
    mpm_status st = MPM_OK;
    auto alloc = [&](void **p, size_t bytes) {
        if (st != MPM_OK) return;
        cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
        if (e != cudaSuccess) st = MPM_ERR_OOM;
    };
    alloc((void **)&c->d_iprop, sizeof(int) * c->nmat);
    alloc((void **)&c->d_matprop, sizeof(double) * 3 * c->nmat);
    alloc((void **)&c->d_matpropf, sizeof(float) * 3 * c->nmat);
    alloc((void **)&c->d_acc, sizeof(unsigned long long) * NACC * N);
    alloc((void **)&c->d_acc2, sizeof(unsigned long long) * 3 * N);
    if (c->fbar) alloc((void **)&c->d_facc, sizeof(unsigned long long) * N);
    alloc(&c->d_nodal, c->rsize * 13 * N);
    alloc((void **)&c->d_nvol, sizeof(double) * N);
    alloc((void **)&c->d_bcflag, N);
    alloc(&c->d_bcval, c->rsize * 3 * N);
    alloc((void **)&c->d_tileflag, g.ntiles);
    alloc((void **)&c->d_eu_part, sizeof(double) * g.ntiles);
    alloc((void **)&c->d_tcount, sizeof(int) * g.nbricks);
    alloc((void **)&c->d_tstart, sizeof(int) * (g.nbricks + 1));
    alloc((void **)&c->d_tcursor, sizeof(int) * g.nbricks);
    alloc((void **)&c->d_scanpart, sizeof(int) * 3 * ((size_t)(g.nbricks + SCAN_SEG - 1) / SCAN_SEG + 1));
    alloc((void **)&c->d_cstart, sizeof(int) * (size_t)g.nbricks * (BRC + 1));
    alloc((void **)&c->d_nwork, sizeof(int));
    alloc((void **)&c->d_blist, sizeof(int) * g.nbricks);
    alloc((void **)&c->d_nblist, sizeof(int));
    alloc((void **)&c->d_tlist, sizeof(int) * g.ntiles);
    alloc((void **)&c->d_ntlist, sizeof(int));
    alloc((void **)&c->d_ctl, sizeof(DevCtl));
    if (st == MPM_OK && cudaMallocHost((void **)&c->h_ctl, sizeof(DevCtl)) != cudaSuccess) st = MPM_ERR_OOM;
    if (st != MPM_OK) {
        mpm_gpu_destroy(c);
        return st;
    }
    cudaMemcpy(c->d_iprop, mat->iprop, sizeof(int) * c->nmat, cudaMemcpyHostToDevice);
    for (int k = 0; k < c->nmat; k++) c->sigma_in = c->sigma_in || mat->iprop[k] == 0;
    {   // a Tait fluid needs only J of its deformation gradient (the FP32 linear explicit path)
        bool all_tait = true;
        for (int k = 0; k < c->nmat; k++) all_tait = all_tait && mat->iprop[k] == 4;
        c->fluid_j = all_tait && c->precision == 32 && !cfg->implicit && !c->affine && !c->fbar &&
                     g.order[0] == 1 && g.order[1] == 1 && g.order[2] == 1;
    }
    cudaMemcpy(c->d_matprop, mat->mat_prop, sizeof(double) * 3 * c->nmat, cudaMemcpyHostToDevice);
    {   // the FP32 kernels read the table without FP64 loads and conversions per particle
        std::vector<float> mf(3 * (size_t)c->nmat);
        for (size_t k = 0; k < mf.size(); k++) mf[k] = (float)mat->mat_prop[k];
        cudaMemcpy(c->d_matpropf, mf.data(), sizeof(float) * mf.size(), cudaMemcpyHostToDevice);
    }
    cudaMemset(c->d_acc, 0, sizeof(unsigned long long) * NACC * N);
    cudaMemset(c->d_acc2, 0, sizeof(unsigned long long) * 3 * N);
    if (c->d_facc) cudaMemset(c->d_facc, 0, sizeof(unsigned long long) * N);
    cudaMemset(c->d_nodal, 0, c->rsize * 13 * N);
    cudaMemset(c->d_bcflag, 0, N);
    cudaMemset(c->d_bcval, 0, c->rsize * 3 * N);
    cudaMemset(c->d_tileflag, 0, g.ntiles);
    cudaMemset(c->d_eu_part, 0, sizeof(double) * g.ntiles);
    cudaMemset(c->d_tcount, 0, sizeof(int) * g.nbricks);
    cudaMemset(c->d_tcursor, 0, sizeof(int) * g.nbricks);
    cudaMemset(c->d_cstart, 0, sizeof(int) * (size_t)g.nbricks * (BRC + 1));
    cudaMemset(c->d_nwork, 0, sizeof(int));
    cudaMemset(c->d_nblist, 0, sizeof(int));
    cudaMemset(c->d_ntlist, 0, sizeof(int));
    cudaMemset(c->d_ctl, 0, sizeof(DevCtl));
    memset(c->h_ctl, 0, sizeof(DevCtl));
    compute_nodal_volume(c);
    if (cudaDeviceSynchronize() != cudaSuccess || check_launch(c) != MPM_OK) {
        mpm_gpu_destroy(c);
        return MPM_ERR_CUDA;
    }
    *out = c;
    return MPM_OK;
}

void mpm_gpu_destroy(mpm_ctx *c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (cudaStream_t st : {c->io_h2d, c->io_d2h})
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    for (cudaEvent_t e : c->io_ev)
        if (e) cudaEventDestroy(e);
    drop_graph(c);
    implicit_free(c);
    free_particles(c);
    free_dev(c->d_iprop);
    free_dev(c->d_matprop);
    free_dev(c->d_matpropf);
    free_dev(c->d_acc);
    free_dev(c->d_acc2);
    free_dev(c->d_facc);
    free_dev(c->d_nodal);
    free_dev(c->d_nvol);
    free_dev(c->d_bcflag);
    free_dev(c->d_bcval);
    free_dev(c->d_tileflag);
    free_dev(c->d_eu_part);
    free_dev(c->d_tcount);
    free_dev(c->d_tstart);
    free_dev(c->d_tcursor);
    free_dev(c->d_scanpart);
    free_dev(c->d_cstart);
    free_dev(c->d_nwork);
    free_dev(c->d_blist);
    free_dev(c->d_nblist);
    free_dev(c->d_tlist);
    free_dev(c->d_ntlist);
    free_dev(c->d_ctl);
    if (c->h_ctl) cudaFreeHost(c->h_ctl);
    for (auto e : c->timer.ev) cudaEventDestroy(e);
    delete c;
}

mpm_status mpm_gpu_set_stream(mpm_ctx *c, void *stream) {
    if (!c) return MPM_ERR_BAD_ARG;
    c->stream = (cudaStream_t)stream;
    return MPM_OK;
}

template <typename R>
static mpm_status upload_particles(mpm_ctx *c, int64_t n, const double *coord, const double *vel, const double *mass,
                                   const double *vol0, const double *F, const double *stress, const int *matid) {
    size_t N = (size_t)n;
    const size_t S = c->pstride;
    const int nr = c->nreal;
    size_t bytes = S * (nr * sizeof(R) + 2 * sizeof(int));
    std::vector<char> host(bytes, 0);
    R *f = (R *)host.data();
    double vmax = 0.0, volmax = 0.0, vsmax = 0.0, mmax = 0.0;
    for (size_t p = 0; p < N; p++) {
        for (int k = 0; k < 3; k++) {
            f[k * S + p] = (R)coord[3 * p + k];
            double v = vel ? vel[3 * p + k] : 0.0;
            f[(3 + k) * S + p] = (R)v;
            vmax = fmax(vmax, fabs(v));
        }
        for (int k = 0; k < 9; k++) {
            // FP32 stores the displacement gradient H = F - I; FP64 stores F
            const double eye = (k % 4) == 0 ? 1.0 : 0.0;
            const double Fk = F ? F[9 * p + k] : eye;
            f[(6 + k) * S + p] = sizeof(R) == 4 ? (R)(Fk - eye) : (R)Fk;
        }
        if (c->fluid_j) {   // J - 1 in field 6, the rest unused
            double H[9];
            for (int k = 0; k < 9; k++) H[k] = F ? F[9 * p + k] - ((k % 4) == 0 ? 1.0 : 0.0) : 0.0;
            f[6 * S + p] = (R)det_ipm1_d(H);
            for (int k = 1; k < 9; k++) f[(6 + k) * S + p] = (R)0;
        }
        double s[6];
        for (int k = 0; k < 6; k++) {
            s[k] = stress ? stress[6 * p + k] : 0.0;
            f[(15 + k) * S + p] = (R)s[k];
        }
        f[21 * S + p] = (R)mass[p];
        f[22 * S + p] = (R)vol0[p];
        f[23 * S + p] = (R)vol0[p];   // vol = vol0 (solid_data_io.cpp:32)
        mmax = fmax(mmax, fabs(mass[p]));
        volmax = fmax(volmax, fabs(vol0[p]));
        double rs = fmax(fabs(s[0]) + fabs(s[5]) + fabs(s[4]),
                         fmax(fabs(s[5]) + fabs(s[1]) + fabs(s[3]), fabs(s[4]) + fabs(s[3]) + fabs(s[2])));
        vsmax = fmax(vsmax, fabs(vol0[p]) * rs);
        // a non-finite input value refuses the load (x * 0 is NaN exactly for inf and NaN)
        double chk = mass[p] * 0.0 + vol0[p] * 0.0 + rs * 0.0;
        for (int k = 0; k < 3; k++) chk += coord[3 * p + k] * 0.0 + (vel ? vel[3 * p + k] * 0.0 : 0.0);
        if (F)
            for (int k = 0; k < 9; k++) chk += F[9 * p + k] * 0.0;
        if (chk != chk) return MPM_ERR_NONFINITE;
    }
    if (c->fbar && sizeof(R) == 8)   // def_grad_bar = I, det_def_grad_bar = 1 (FP32 stores both minus 1: zeros)
        for (size_t p = 0; p < N; p++) {
            f[(c->off_fbar + 0) * S + p] = f[(c->off_fbar + 4) * S + p] = f[(c->off_fbar + 8) * S + p] = (R)1;
            f[(c->off_fbar + 9) * S + p] = (R)1;
        }
    int *ip = (int *)(f + nr * S);
    for (size_t p = 0; p < N; p++) {
        int mid = matid ? matid[p] : 0;
        if (mid < 0 || mid >= c->nmat) return MPM_ERR_BAD_ARG;
        ip[p] = mid;
        ip[S + p] = (int)p;
    }
    CK(cudaMemcpy(c->pbuf[c->cur], host.data(), bytes, cudaMemcpyHostToDevice));
    c->mmax = mmax * 1.000001;
    // bounds for the first step's fixed-point scales (slot of the current parity)
    DevCtl h;
    memset(&h, 0, sizeof(h));
    int par = (int)(c->step & 1);
    auto fb = [](double v) {
        float f = (float)(v * 1.000001);
        unsigned u;
        memcpy(&u, &f, 4);
        return u;
    };
    h.nxt[par][B_VMAX] = fb(vmax);
    h.nxt[par][B_VOLMAX] = fb(volmax);
    h.nxt[par][B_VOLSMAX] = fb(vsmax);
    CK(cudaMemcpy(c->d_ctl, &h, sizeof(DevCtl), cudaMemcpyHostToDevice));
    return MPM_OK;
}

mpm_status mpm_gpu_load_particles(mpm_ctx *c, int64_t n, const double *coord, const double *vel, const double *mass,
                                  const double *vol0, const double *F, const double *stress, const int *matid) {
    if (!c || n < 0 || n > (1LL << 30) || (n > 0 && (!coord || !mass || !vol0))) return MPM_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(c->stream));
    free_particles(c);
    c->num = n;
    size_t N = (size_t)(n > 0 ? n : 1);
    c->pstride = (N + 63) / 64 * 64;
    size_t bytes = c->pstride * (c->nreal * c->rsize + 2 * sizeof(int));
    CK(cudaMalloc(&c->pbuf[0], bytes));
    CK(cudaMalloc(&c->pbuf[1], bytes));
    CK(cudaMalloc((void **)&c->d_key, sizeof(int) * N));
    CK(cudaMalloc((void **)&c->d_perm, sizeof(int) * N));
    CK(cudaMalloc((void **)&c->d_tmp, sizeof(int) * N));
    CK(cudaMalloc((void **)&c->d_perm2, sizeof(int) * N));
    c->nwork_cap = c->g.nbricks + (int)(N / CHUNK) + 1;
    CK(cudaMalloc((void **)&c->d_work, sizeof(WorkItem) * c->nwork_cap));
    c->cur = 0;
    mpm_status s = c->precision == 64 ? upload_particles<double>(c, n, coord, vel, mass, vol0, F, stress, matid)
                                      : upload_particles<float>(c, n, coord, vel, mass, vol0, F, stress, matid);
    if (s != MPM_OK) {   // a refused load leaves the context without particles
        free_particles(c);
        return s;
    }
    CK(cudaMemset(c->d_acc, 0, sizeof(unsigned long long) * NACC * c->g.nodec));
    CK(cudaMemset(c->d_acc2, 0, sizeof(unsigned long long) * 3 * c->g.nodec));
    CK(cudaMemset(c->d_tileflag, 0, c->g.ntiles));
    c->accum_dirty = false;
    c->stage = 0;
    if (n > 0) {
        s = sort_particles(c);
        if (s != MPM_OK) return s;
    }
    CK(cudaStreamSynchronize(c->stream));
    return MPM_OK;
}

mpm_status mpm_gpu_set_bc(mpm_ctx *c, int comp, int n, const int *nodes, const double *vals) {
    if (!c || comp < 0 || comp > 2 || n < 0 || (n > 0 && (!nodes || !vals))) return MPM_ERR_BAD_ARG;
    for (int i = 0; i < n; i++)
        if (nodes[i] < 0 || nodes[i] >= c->g.nodec) return MPM_ERR_BAD_ARG;
    c->bc_nodes[comp].assign(nodes, nodes + n);
    c->bc_vals[comp].assign(vals, vals + n);
    size_t N = (size_t)c->g.nodec;
    std::vector<unsigned char> flag(N, 0);
    std::vector<double> val(3 * N, 0.0);
    for (int k = 0; k < 3; k++)
        for (size_t i = 0; i < c->bc_nodes[k].size(); i++) {   // later entries win, as BCSetVal's loop
            int nd = c->bc_nodes[k][i];
            flag[nd] |= (unsigned char)(1 << k);
            val[k * N + nd] = c->bc_vals[k][i];
        }
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(c->d_bcflag, flag.data(), N, cudaMemcpyHostToDevice));
    if (c->precision == 64) {
        CK(cudaMemcpy(c->d_bcval, val.data(), sizeof(double) * 3 * N, cudaMemcpyHostToDevice));
    } else {
        std::vector<float> vf(3 * N);
        for (size_t i = 0; i < 3 * N; i++) vf[i] = (float)val[i];
        CK(cudaMemcpy(c->d_bcval, vf.data(), sizeof(float) * 3 * N, cudaMemcpyHostToDevice));
    }
    if (c->imp) return implicit_bc_changed(c);
    return MPM_OK;
}

static mpm_status begin_step(mpm_ctx *c, double facl) {
    if (c->accum_dirty) {
        CK(cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * NACC * c->g.nodec, c->stream));
        CK(cudaMemsetAsync(c->d_acc2, 0, sizeof(unsigned long long) * 3 * c->g.nodec, c->stream));
        CK(cudaMemsetAsync(c->d_tileflag, 0, c->g.ntiles, c->stream));
        c->accum_dirty = false;
    }
    if (c->steps_since_sort >= c->resort_period) {
        mpm_status s = sort_particles(c);
        if (s != MPM_OK) return s;
    }
    mpm_status s = run_p2g(c, facl);
    if (s != MPM_OK) return s;
    return run_grid1(c, 0);
}

mpm_status mpm_gpu_p2g(mpm_ctx *c, double facl) {
    if (!c) return MPM_ERR_BAD_ARG;
    if (c->num == 0) return MPM_ERR_STATE;
    c->write_nodal_dl = true;
    if (c->stage != 0) c->accum_dirty = true;
    mpm_status s = begin_step(c, facl);
    c->stage = 1;
    return s;
}

mpm_status mpm_gpu_grid_update(mpm_ctx *c) {
    // SolveSolid's a = f/m with the BC zeroing is evaluated in the same grid
    // pass as Particle2NodeS's nvel; this call only checks the ordering.
    if (!c) return MPM_ERR_BAD_ARG;
    if (c->stage != 1) return MPM_ERR_STATE;
    c->stage = 2;
    return MPM_OK;
}

mpm_status mpm_gpu_g2p(mpm_ctx *c) {
    if (!c) return MPM_ERR_BAD_ARG;
    if (c->stage != 2) return MPM_ERR_STATE;
    c->write_nodal_dl = true;
    mpm_status s = run_g2p(c);
    c->accum_dirty = true;   // accumulators kept for downloads; cleared by the next P2G
    c->stage = 0;
    c->step++;
    c->steps_since_sort++;
    return s;
}

static mpm_status eager_steps(mpm_ctx *c, int nsteps, double facl) {
    for (int s = 0; s < nsteps; s++) {
        mpm_status st = begin_step(c, facl);
        if (st != MPM_OK) return st;
        st = run_g2p(c);
        if (st != MPM_OK) return st;
        c->step++;
        c->steps_since_sort++;
    }
    return MPM_OK;
}

void drop_graph(mpm_ctx *c) {
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
}

// Captures G = 2 * resort_period fused steps, starting at a step with a
// re-sort due and even step parity, into one executable graph.  Two re-sorts
// per block leave the particle buffers where they were and an even step
// count leaves the bound-slot parity unchanged, so the same graph replays
// every block.  Launch configurations never depend on device data, so the
// host-side bookkeeping of a replay is the same as that of the captured steps.
static mpm_status capture_block(mpm_ctx *c, int G, double facl) {
    drop_graph(c);
    const int64_t l0 = c->launches;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    mpm_status st = eager_steps(c, G, facl);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (st != MPM_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return st != MPM_OK ? st : MPM_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&c->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->graph_exec = nullptr;
        return MPM_ERR_CUDA;
    }
    c->graph_launches = c->launches - l0;
    c->graph_facl = facl;
    c->graph_stream = c->stream;
    c->graph_tune = c->tune;
    c->graph_cur = c->cur;
    c->graph_pbuf[0] = c->pbuf[0];
    c->graph_pbuf[1] = c->pbuf[1];
    // the captured steps have not run yet: the first launch runs them
    CK(cudaGraphLaunch(c->graph_exec, c->stream));
    c->graph_replays++;
    return MPM_OK;
}

mpm_status mpm_gpu_step_explicit(mpm_ctx *c, int nsteps, double facl) {
    if (!c || nsteps < 0) return MPM_ERR_BAD_ARG;
    if (c->num == 0) return MPM_ERR_STATE;
    if (c->stage != 0) return MPM_ERR_STATE;
    c->write_nodal_dl = false;
    const int G = 2 * c->resort_period;
    if (!c->use_graph || c->stream == nullptr || c->timer.on || nsteps < 3 * G) return eager_steps(c, nsteps, facl);
    int done = 0;
    while (done < nsteps && !(c->steps_since_sort >= c->resort_period && (c->step & 1) == 0)) {
        mpm_status st = eager_steps(c, 1, facl);
        if (st != MPM_OK) return st;
        done++;
    }
    if (c->graph_exec && (c->graph_facl != facl || c->graph_stream != c->stream ||
                          !mpm::same_launches(c->graph_tune, c->tune) ||
                          c->graph_cur != c->cur ||
                          c->graph_pbuf[0] != c->pbuf[0] || c->graph_pbuf[1] != c->pbuf[1]))
        drop_graph(c);
    if (!c->graph_exec && nsteps - done >= G) {
        mpm_status st = capture_block(c, G, facl);
        if (st != MPM_OK) return st;
        done += G;
    }
    while (c->graph_exec && nsteps - done >= G) {
        CK(cudaGraphLaunch(c->graph_exec, c->stream));
        c->step += G;
        c->resorts += 2;
        c->steps_since_sort = c->resort_period;
        c->launches += c->graph_launches;
        c->graph_replays++;
        done += G;
    }
    return eager_steps(c, nsteps - done, facl);
}

mpm_status mpm_gpu_set_graph(mpm_ctx *c, int on) {
    if (!c) return MPM_ERR_BAD_ARG;
    c->use_graph = on != 0;
    if (!c->use_graph) drop_graph(c);
    return MPM_OK;
}

static mpm_status read_errors(mpm_ctx *c) {
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(c->h_ctl, c->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost));
    if (c->latched != MPM_OK) return c->latched;
    if (c->h_ctl->err_timeout) return MPM_ERR_DEVICE_TIMEOUT;
    if (c->h_ctl->err_nonfinite) return MPM_ERR_NONFINITE;
    if (c->h_ctl->err_oob) return MPM_ERR_PARTICLE_OUT_OF_BOX;
    return MPM_OK;
}

mpm_status mpm_gpu_sync(mpm_ctx *c) {
    if (!c) return MPM_ERR_BAD_ARG;
    mpm_status s = read_errors(c);
    if (s != MPM_OK && s != MPM_ERR_CUDA) {
        // clear latched device error counters
        unsigned z[2] = {0, 0};
        cudaMemcpy(&c->d_ctl->err_oob, z, sizeof(unsigned) * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(&c->d_ctl->err_timeout, z, sizeof(unsigned), cudaMemcpyHostToDevice);
        c->latched = MPM_OK;
    }
    return s;
}

template <typename R>
static void to_host(const void *dev, size_t count, double *host) {
    std::vector<R> t(count);
    cudaMemcpy(t.data(), dev, sizeof(R) * count, cudaMemcpyDeviceToHost);
    for (size_t i = 0; i < count; i++) host[i] = (double)t[i];
}

mpm_status mpm_gpu_download_nodal(mpm_ctx *c, int field, double *host) {
    if (!c || !host || field < 0 || field > 6) return MPM_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(c->stream));
    size_t N = (size_t)c->g.nodec;
    if (field == 6) {
        CK(cudaMemcpy(host, c->d_nvol, sizeof(double) * N, cudaMemcpyDeviceToHost));
        return MPM_OK;
    }
    if (field == 4 || field == 5) {
        // nvel: after g2p the MUSL velocity, before it the P2G velocity; naccel from the grid update
        size_t off = (field == 5) ? 10 * N : (c->stage == 0 && c->step > 0 ? 4 * N : 7 * N);
        const char *base = (const char *)c->d_nodal + off * c->rsize;
        if (c->precision == 64) to_host<double>(base, 3 * N, host);
        else to_host<float>(base, 3 * N, host);
        return MPM_OK;
    }
    // accumulated sums, with the scales the last P2G used
    std::vector<long long> q;
    DevCtl h;
    CK(cudaMemcpy(&h, c->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost));
    int f0 = field == 0 ? 0 : field == 1 ? 1 : field == 2 ? 2 : 5;
    int nf = (field <= 1) ? 1 : 3;
    const double inv = h.p2g_inv[field == 0 ? 0 : field == 1 ? 1 : field == 2 ? 2 : 3];
    q.resize(nf * N);
    CK(cudaMemcpy(q.data(), c->d_acc + (size_t)f0 * N, sizeof(long long) * nf * N, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < nf * N; i++) {
        double v = (double)q[i] * inv;
        if (c->precision == 32) v = (double)(float)v;
        host[i] = v;
    }
    if (field == 1)
        for (size_t i = 0; i < N; i++)
            if (host[i] < c->mtol) host[i] = 0.0;   // Particle2NodeS:88
    return MPM_OK;
}

// Host <-> device particle state in the reference's FP64 AoS layout.  The
// copies go through a device staging buffer in load order; a kernel moves the
// fields between it and the sorted SoA arrays (pid maps sorted -> load index).
// Staging layout (per particle, load order): coord 3 | vel 3 | F 9 | stress 6 | vol 1.
namespace mpm {
constexpr int ST_X = 0, ST_V = 3, ST_F = 6, ST_S = 15, ST_VOL = 21, ST_W = 22;

template <typename R>
__global__ void k_state_gather(const R *__restrict__ f, size_t N, size_t S, int nreal, double *__restrict__ st,
                               unsigned mask, int fluidj = 0) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const int *pid = (const int *)(f + nreal * S) + S;
    const size_t p = (size_t)pid[j];
    if (mask & 1)
        for (int k = 0; k < 3; k++) st[ST_X * N + 3 * p + k] = (double)f[k * S + j];
    if (mask & 2)
        for (int k = 0; k < 3; k++) st[ST_V * N + 3 * p + k] = (double)f[(3 + k) * S + j];
    if ((mask & 4) && fluidj) {   // only J is kept: F = J^(1/3) I
        const double c3 = cbrt(1.0 + (double)f[6 * S + j]);
        for (int k = 0; k < 9; k++) st[ST_F * N + 9 * p + k] = (k % 4) == 0 ? c3 : 0.0;
    } else if (mask & 4) {
        for (int k = 0; k < 9; k++)
            st[ST_F * N + 9 * p + k] = (double)f[(6 + k) * S + j] + (sizeof(R) == 4 && (k % 4) == 0 ? 1.0 : 0.0);
    }
    if (mask & 8)
        for (int k = 0; k < 6; k++) st[ST_S * N + 6 * p + k] = (double)f[(15 + k) * S + j];
    if (mask & 16) st[ST_VOL * N + p] = (double)f[23 * S + j];
}

// Also raises the fixed-point bounds of the next P2G to cover the new state.
template <typename R>
__global__ void k_state_scatter(R *__restrict__ f, size_t N, size_t S, int nreal, const double *__restrict__ st,
                                unsigned mask, DevCtl *ctl, int parity, int fluidj = 0) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    {
        const size_t p = (size_t)((const int *)(f + nreal * S) + S)[j];
        if (mask & 2) {
            float vm = 0.0f;
            for (int k = 0; k < 3; k++) vm = fmaxf(vm, fabsf((float)st[ST_V * N + 3 * p + k]));
            atomic_max_pos(&ctl->nxt[parity][B_VMAX], vm * 1.000001f);
        }
        const float vol = (mask & 16) ? fabsf((float)st[ST_VOL * N + p]) : fabsf((float)f[23 * S + j]);
        if (mask & 16) atomic_max_pos(&ctl->nxt[parity][B_VOLMAX], vol * 1.000001f);
        if (mask & 8) {
            const double *s6 = st + ST_S * N + 6 * p;
            const double rs = fmax(fabs(s6[0]) + fabs(s6[5]) + fabs(s6[4]),
                                   fmax(fabs(s6[5]) + fabs(s6[1]) + fabs(s6[3]), fabs(s6[4]) + fabs(s6[3]) + fabs(s6[2])));
            atomic_max_pos(&ctl->nxt[parity][B_VOLSMAX], (float)(vol * rs) * 1.000001f);
        }
    }
    const int *pid = (const int *)(f + nreal * S) + S;
    const size_t p = (size_t)pid[j];
    {   // a non-finite value from the host is reported by the next synchronising call
        double chk = 0.0;
        if (mask & 1)
            for (int k = 0; k < 3; k++) chk += st[ST_X * N + 3 * p + k] * 0.0;
        if (mask & 2)
            for (int k = 0; k < 3; k++) chk += st[ST_V * N + 3 * p + k] * 0.0;
        if (mask & 4)
            for (int k = 0; k < 9; k++) chk += st[ST_F * N + 9 * p + k] * 0.0;
        if (mask & 8)
            for (int k = 0; k < 6; k++) chk += st[ST_S * N + 6 * p + k] * 0.0;
        if (mask & 16) chk += st[ST_VOL * N + p] * 0.0;
        if (chk != 0.0 || chk != chk) atomicAdd(&ctl->err_nonfinite, 1u);   // x * 0 is NaN for inf and NaN
    }
    if (mask & 1)
        for (int k = 0; k < 3; k++) f[k * S + j] = (R)st[ST_X * N + 3 * p + k];
    if (mask & 2)
        for (int k = 0; k < 3; k++) f[(3 + k) * S + j] = (R)st[ST_V * N + 3 * p + k];
    if ((mask & 4) && fluidj) {   // only J - 1 is kept
        double H[9];
        for (int k = 0; k < 9; k++) H[k] = st[ST_F * N + 9 * p + k] - ((k % 4) == 0 ? 1.0 : 0.0);
        f[6 * S + j] = (R)det_ipm1_d(H);
    } else if (mask & 4) {
        for (int k = 0; k < 9; k++)
            f[(6 + k) * S + j] = (R)(st[ST_F * N + 9 * p + k] - (sizeof(R) == 4 && (k % 4) == 0 ? 1.0 : 0.0));
    }
    if (mask & 8)
        for (int k = 0; k < 6; k++) f[(15 + k) * S + j] = (R)st[ST_S * N + 6 * p + k];
    if (mask & 16) f[23 * S + j] = (R)st[ST_VOL * N + p];
}
// The affine matrices from the staging buffer (load order) into fields
// 24..32; raises the next P2G's momentum bound to max_c (|v_c| + sum_j |A_cj| dmax_j).
template <typename R>
__global__ void k_affine_scatter_state(R *f, size_t N, size_t S, int nreal, const double *st, DevCtl *ctl, int parity,
                                       double d0, double d1, double d2) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const size_t p = (size_t)((const int *)(f + nreal * S) + S)[j];
    float bm = 0.0f;
    double chk = 0.0;
    for (int c = 0; c < 3; c++) {
        double b = fabs((double)f[(3 + c) * S + j]);
        const double dm[3] = {d0, d1, d2};
        for (int k = 0; k < 3; k++) {
            const double v = st[9 * p + 3 * c + k];
            f[(24 + 3 * c + k) * S + j] = (R)v;
            b += fabs(v) * dm[k];
            chk += v * 0.0;
        }
        bm = fmaxf(bm, (float)b);
    }
    if (chk != chk) atomicAdd(&ctl->err_nonfinite, 1u);
    if (bm > 0.0f) atomic_max_pos(&ctl->nxt[parity][B_VMAX], bm * 1.000001f);
}

// def_grad_bar and det_def_grad_bar into the staging buffer in load order.
template <typename R>
__global__ void k_fbar_gather_state(const R *f, size_t N, size_t S, int nreal, int off, double *st) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const size_t p = (size_t)((const int *)(f + nreal * S) + S)[j];
    for (int k = 0; k < 9; k++)
        st[9 * p + k] = (double)f[(off + k) * S + j] + (sizeof(R) == 4 && (k % 4) == 0 ? 1.0 : 0.0);
    st[9 * N + p] = (double)f[(off + 9) * S + j] + (sizeof(R) == 4 ? 1.0 : 0.0);
}

// The affine matrices (fields 24..32) into the staging buffer in load order.
template <typename R>
__global__ void k_affine_gather_state(const R *f, size_t N, size_t S, int nreal, double *st) {
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const size_t p = (size_t)((const int *)(f + nreal * S) + S)[j];
    for (int k = 0; k < 9; k++) st[9 * p + k] = (double)f[(24 + k) * S + j];
}
}  // namespace mpm

static mpm_status ensure_staging(mpm_ctx *c) {
    if (c->d_stage) return MPM_OK;
    CK(cudaMalloc((void **)&c->d_stage, sizeof(double) * ST_W * (size_t)c->num));
    return MPM_OK;
}

mpm_status mpm_gpu_download_particles(mpm_ctx *c, double *coord, double *vel, double *F, double *stress, double *vol) {
    if (!c) return MPM_ERR_BAD_ARG;
    if (c->num == 0) return MPM_OK;
    mpm_status s = ensure_staging(c);
    if (s != MPM_OK) return s;
    const size_t N = (size_t)c->num;
    unsigned mask = (coord ? 1u : 0u) | (vel ? 2u : 0u) | (F ? 4u : 0u) | (stress ? 8u : 0u) | (vol ? 16u : 0u);
    const int nb = (int)((N + 255) / 256);
    if (c->precision == 64) k_state_gather<double><<<nb, 256, 0, c->stream>>>((const double *)c->pbuf[c->cur], N, c->pstride, c->nreal, c->d_stage, mask);
    else k_state_gather<float><<<nb, 256, 0, c->stream>>>((const float *)c->pbuf[c->cur], N, c->pstride, c->nreal, c->d_stage, mask, c->fluid_j);
    c->launches++;
    if (check_launch(c) != MPM_OK) return MPM_ERR_CUDA;
    const double *st = c->d_stage;
    if (coord) CK(cudaMemcpyAsync(coord, st + ST_X * N, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, c->stream));
    if (vel) CK(cudaMemcpyAsync(vel, st + ST_V * N, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, c->stream));
    if (F) CK(cudaMemcpyAsync(F, st + ST_F * N, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, c->stream));
    if (stress) CK(cudaMemcpyAsync(stress, st + ST_S * N, sizeof(double) * 6 * N, cudaMemcpyDeviceToHost, c->stream));
    if (vol) CK(cudaMemcpyAsync(vol, st + ST_VOL * N, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return MPM_OK;
}

mpm_status mpm_gpu_download_affine(mpm_ctx *c, double *affine) {
    if (!c || (!affine && c->num > 0)) return MPM_ERR_BAD_ARG;
    if (c->num == 0) return MPM_OK;
    const size_t N = (size_t)c->num;
    if (!c->affine) {
        memset(affine, 0, sizeof(double) * 9 * N);
        return MPM_OK;
    }
    mpm_status s = ensure_staging(c);
    if (s != MPM_OK) return s;
    const int nb = (int)((N + 255) / 256);
    if (c->precision == 64)
        k_affine_gather_state<double><<<nb, 256, 0, c->stream>>>((const double *)c->pbuf[c->cur], N, c->pstride,
                                                                  c->nreal, c->d_stage);
    else
        k_affine_gather_state<float><<<nb, 256, 0, c->stream>>>((const float *)c->pbuf[c->cur], N, c->pstride,
                                                                 c->nreal, c->d_stage);
    c->launches++;
    if (check_launch(c) != MPM_OK) return MPM_ERR_CUDA;
    CK(cudaMemcpyAsync(affine, c->d_stage, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return MPM_OK;
}

mpm_status mpm_gpu_download_fbar(mpm_ctx *c, double *Fbar, double *Jbar) {
    if (!c) return MPM_ERR_BAD_ARG;
    if (!c->fbar) return MPM_ERR_STATE;
    if (c->num == 0) return MPM_OK;
    mpm_status s = ensure_staging(c);
    if (s != MPM_OK) return s;
    const size_t N = (size_t)c->num;
    const int nb = (int)((N + 255) / 256);
    if (c->precision == 64)
        k_fbar_gather_state<double><<<nb, 256, 0, c->stream>>>((const double *)c->pbuf[c->cur], N, c->pstride,
                                                                c->nreal, c->off_fbar, c->d_stage);
    else
        k_fbar_gather_state<float><<<nb, 256, 0, c->stream>>>((const float *)c->pbuf[c->cur], N, c->pstride,
                                                               c->nreal, c->off_fbar, c->d_stage);
    c->launches++;
    if (check_launch(c) != MPM_OK) return MPM_ERR_CUDA;
    if (Fbar) CK(cudaMemcpyAsync(Fbar, c->d_stage, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, c->stream));
    if (Jbar) CK(cudaMemcpyAsync(Jbar, c->d_stage + 9 * N, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return MPM_OK;
}

mpm_status mpm_gpu_upload_affine(mpm_ctx *c, const double *affine) {
    if (!c || (!affine && c->num > 0)) return MPM_ERR_BAD_ARG;
    if (!c->affine) return MPM_ERR_STATE;
    if (c->num == 0) return MPM_OK;
    mpm_status s = ensure_staging(c);
    if (s != MPM_OK) return s;
    const size_t N = (size_t)c->num;
    CK(cudaMemcpyAsync(c->d_stage, affine, sizeof(double) * 9 * N, cudaMemcpyHostToDevice, c->stream));
    double dm[3];
    for (int d = 0; d < 3; d++) dm[d] = (c->g.order[d] == 2 ? 1.5 : 1.0) * c->g.dx[d];
    const int nb = (int)((N + 255) / 256), par = (int)(c->step & 1);
    if (c->precision == 64)
        k_affine_scatter_state<double><<<nb, 256, 0, c->stream>>>((double *)c->pbuf[c->cur], N, c->pstride, c->nreal,
                                                                   c->d_stage, c->d_ctl, par, dm[0], dm[1], dm[2]);
    else
        k_affine_scatter_state<float><<<nb, 256, 0, c->stream>>>((float *)c->pbuf[c->cur], N, c->pstride, c->nreal,
                                                                  c->d_stage, c->d_ctl, par, dm[0], dm[1], dm[2]);
    c->launches++;
    if (check_launch(c) != MPM_OK) return MPM_ERR_CUDA;
    CK(cudaStreamSynchronize(c->stream));
    return MPM_OK;
}

mpm_status mpm_gpu_upload_particles(mpm_ctx *c, const double *coord, const double *vel, const double *F,
                                    const double *stress, const double *vol) {
    if (!c) return MPM_ERR_BAD_ARG;
    if (c->num == 0) return MPM_OK;
    mpm_status s = ensure_staging(c);
    if (s != MPM_OK) return s;
    const size_t N = (size_t)c->num;
    double *st = c->d_stage;
    if (coord) CK(cudaMemcpyAsync(st + ST_X * N, coord, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, c->stream));
    if (vel) CK(cudaMemcpyAsync(st + ST_V * N, vel, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, c->stream));
    if (F) CK(cudaMemcpyAsync(st + ST_F * N, F, sizeof(double) * 9 * N, cudaMemcpyHostToDevice, c->stream));
    if (stress) CK(cudaMemcpyAsync(st + ST_S * N, stress, sizeof(double) * 6 * N, cudaMemcpyHostToDevice, c->stream));
    if (vol) CK(cudaMemcpyAsync(st + ST_VOL * N, vol, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    unsigned mask = (coord ? 1u : 0u) | (vel ? 2u : 0u) | (F ? 4u : 0u) | (stress ? 8u : 0u) | (vol ? 16u : 0u);
    const int nb = (int)((N + 255) / 256);
    const int par = (int)(c->step & 1);
    if (c->precision == 64)
        k_state_scatter<double><<<nb, 256, 0, c->stream>>>((double *)c->pbuf[c->cur], N, c->pstride, c->nreal, st, mask, c->d_ctl, par);
    else
        k_state_scatter<float><<<nb, 256, 0, c->stream>>>((float *)c->pbuf[c->cur], N, c->pstride, c->nreal, st, mask, c->d_ctl, par, c->fluid_j);
    c->launches++;
    return check_launch(c);
}

// Explicit steps with the particle state read from and written back to host
// arrays every step.  Uploads run on one copy stream, downloads on another,
// in pieces (io_chunks per field, the small fields first): the upload of a
// piece for step n + 1 waits only for the download of the same piece from
// step n, so uploads overlap the remaining downloads and both directions of
// the host link carry data at once.
mpm_status mpm_gpu_steps_host(mpm_ctx *c, int nsteps, double facl, double *coord, double *vel, double *F,
                              double *stress, double *vol) {
    if (!c || nsteps < 0) return MPM_ERR_BAD_ARG;
    if (c->num == 0 || nsteps == 0) return MPM_OK;
    if (c->imp) return MPM_ERR_STATE;
    mpm_status s = ensure_staging(c);
    if (s != MPM_OK) return s;
    const int NC = c->io_chunks;
    constexpr int M = mpm_ctx::IO_MAX_CHUNKS;
    constexpr int EV_UP = 0, EV_DOWN = 5 * M, EV_GATHER = 10 * M, EV_START = 10 * M + 1;
    if (!c->io_h2d) {
        CK(cudaStreamCreateWithFlags(&c->io_h2d, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&c->io_d2h, cudaStreamNonBlocking));
        for (cudaEvent_t &e : c->io_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const size_t N = (size_t)c->num;
    // fields in copy order, smallest first: vol, coord, vel, stress, F
    double *host[5] = {vol, coord, vel, stress, F};
    const int off[5] = {ST_VOL, ST_X, ST_V, ST_S, ST_F}, width[5] = {1, 3, 3, 6, 9};
    const unsigned bit[5] = {16u, 1u, 2u, 8u, 4u};
    unsigned mask = 0;
    for (int f = 0; f < 5; f++)
        if (host[f]) mask |= bit[f];
    double *st = c->d_stage;
    const int nb = (int)((N + 255) / 256);
    auto piece = [&](int f, int k, size_t &begin, size_t &count) {
        const size_t total = (size_t)width[f] * N;
        const size_t per = (total + NC - 1) / NC;
        begin = std::min(total, (size_t)k * per);
        count = std::min(total, begin + per) - begin;
    };
    // the copy streams start after the work already on the context's stream
    CK(cudaEventRecord(c->io_ev[EV_START], c->stream));
    CK(cudaStreamWaitEvent(c->io_h2d, c->io_ev[EV_START], 0));
    CK(cudaStreamWaitEvent(c->io_d2h, c->io_ev[EV_START], 0));
    for (int step = 0; step < nsteps; step++) {
        for (int f = 0; f < 5; f++) {
            if (!host[f]) continue;
            for (int k = 0; k < NC; k++) {
                size_t b0, cnt;
                piece(f, k, b0, cnt);
                if (cnt == 0) continue;
                if (step > 0) CK(cudaStreamWaitEvent(c->io_h2d, c->io_ev[EV_DOWN + f * M + k], 0));
                CK(cudaMemcpyAsync(st + (size_t)off[f] * N + b0, host[f] + b0, sizeof(double) * cnt,
                                   cudaMemcpyHostToDevice, c->io_h2d));
                CK(cudaEventRecord(c->io_ev[EV_UP + f * M + k], c->io_h2d));
                CK(cudaStreamWaitEvent(c->stream, c->io_ev[EV_UP + f * M + k], 0));
            }
        }
        const int par = (int)(c->step & 1);
        if (c->precision == 64)
            k_state_scatter<double><<<nb, 256, 0, c->stream>>>((double *)c->pbuf[c->cur], N, c->pstride, c->nreal, st,
                                                                mask, c->d_ctl, par);
        else
            k_state_scatter<float><<<nb, 256, 0, c->stream>>>((float *)c->pbuf[c->cur], N, c->pstride, c->nreal, st,
                                                               mask, c->d_ctl, par, c->fluid_j);
        c->launches++;
        if ((s = check_launch(c)) != MPM_OK) return s;
        if ((s = mpm_gpu_step_explicit(c, 1, facl)) != MPM_OK) return s;
        if (c->precision == 64)
            k_state_gather<double><<<nb, 256, 0, c->stream>>>((const double *)c->pbuf[c->cur], N, c->pstride,
                                                               c->nreal, st, mask);
        else
            k_state_gather<float><<<nb, 256, 0, c->stream>>>((const float *)c->pbuf[c->cur], N, c->pstride,
                                                              c->nreal, st, mask, c->fluid_j);
        c->launches++;
        if ((s = check_launch(c)) != MPM_OK) return s;
        CK(cudaEventRecord(c->io_ev[EV_GATHER], c->stream));
        CK(cudaStreamWaitEvent(c->io_d2h, c->io_ev[EV_GATHER], 0));
        for (int f = 0; f < 5; f++) {
            if (!host[f]) continue;
            for (int k = 0; k < NC; k++) {
                size_t b0, cnt;
                piece(f, k, b0, cnt);
                if (cnt == 0) continue;
                CK(cudaMemcpyAsync(host[f] + b0, st + (size_t)off[f] * N + b0, sizeof(double) * cnt,
                                   cudaMemcpyDeviceToHost, c->io_d2h));
                CK(cudaEventRecord(c->io_ev[EV_DOWN + f * M + k], c->io_d2h));
            }
        }
    }
    CK(cudaStreamSynchronize(c->io_d2h));
    CK(cudaStreamSynchronize(c->stream));
    return MPM_OK;
}

mpm_status mpm_gpu_get_stats(mpm_ctx *c, mpm_stats *out) {
    if (!c || !out) return MPM_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(c->stream));
    DevCtl h;
    CK(cudaMemcpy(&h, c->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost));
    int nw = 0;
    CK(cudaMemcpy(&nw, c->d_nwork, sizeof(int), cudaMemcpyDeviceToHost));
    out->num = c->num;
    out->nodec = c->g.nodec;
    out->steps = c->step;
    out->resorts = c->resorts;
    out->kernel_launches = c->launches;
    out->out_of_box = h.err_oob;
    out->tile_misses = h.tile_misses;
    out->ntiles = c->g.nbricks;
    out->nwork = nw;
    return MPM_OK;
}

// One CTA waits, through the same bounded mbarrier wait the bulk-copy staged
// kernels use, on a barrier that nothing arrives on; the wait gives up after
// limit_ns, the kernel records the timeout as those kernels do and returns.
__global__ void k_selftest_wait(DevCtl *ctl, unsigned long long limit_ns) {
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0u, 1u << 30, limit_ns);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicAdd(&ctl->err_timeout, 1u);
}

mpm_status mpm_gpu_selftest_wait(mpm_ctx *c, double seconds) {
    if (!c || !(seconds > 0.0) || seconds > 1.0) return MPM_ERR_BAD_ARG;
    k_selftest_wait<<<1, 32, 0, c->stream>>>(c->d_ctl, (unsigned long long)(seconds * 1e9));
    CK(cudaGetLastError());
    c->launches++;
    return MPM_OK;
}

mpm_status mpm_gpu_autotune(mpm_ctx *c, int steps_per_trial, double facl) {
    if (!c || steps_per_trial <= 0) return MPM_ERR_BAD_ARG;
    if (c->num == 0 || c->stage != 0) return MPM_ERR_STATE;
    // every candidate computes bitwise the same step, so the trial steps are
    // ordinary simulation steps; each kernel class is timed on its own
    const int p2g_opts[3] = {2, 3, 2}, stg_opts[3] = {1, 0, 0}, musl_opts[3] = {3, 2, 3}, mstg_opts[3] = {1, 0, 0};
    const int upd_opts[3] = {3, 0, 2};
    double best[3] = {1e300, 1e300, 1e300};
    Tune pick = c->tune;
    const bool was_on = c->timer.on;
    for (int t = 0; t < 3; t++) {
        c->tune.p2g_minb = p2g_opts[t];
        c->tune.p2g_staged = stg_opts[t];
        c->tune.musl_minb = musl_opts[t];
        c->tune.musl_staged = mstg_opts[t];
        c->tune.update_ctas_per_sm = upd_opts[t];
        int cnt = NKCLASS;
        const char *names[NKCLASS];
        double ms[NKCLASS];
        int64_t nl[NKCLASS];
        mpm_gpu_kernel_times(c, &cnt, nullptr, nullptr, nullptr);   // discard earlier records
        c->timer.on = true;
        mpm_status st = mpm_gpu_step_explicit(c, steps_per_trial, facl);
        c->timer.on = was_on;
        if (st != MPM_OK) return st;
        cnt = NKCLASS;
        st = mpm_gpu_kernel_times(c, &cnt, names, ms, nl);
        if (st != MPM_OK) return st;
        if (ms[K_P2G] < best[0]) {
            best[0] = ms[K_P2G];
            pick.p2g_minb = p2g_opts[t];
            pick.p2g_staged = stg_opts[t];
        }
        if (ms[K_G2P_MUSL] < best[1]) {
            best[1] = ms[K_G2P_MUSL];
            pick.musl_minb = musl_opts[t];
            pick.musl_staged = mstg_opts[t];
        }
        if (ms[K_G2P_UPDATE] < best[2]) { best[2] = ms[K_G2P_UPDATE]; pick.update_ctas_per_sm = upd_opts[t]; }
    }
    pick.done = true;
    c->tune = pick;
    return MPM_OK;
}

mpm_status mpm_gpu_set_tuning(mpm_ctx *c, int p2g_minb, int musl_minb, int update_ctas_per_sm) {
    if (!c) return MPM_ERR_BAD_ARG;
    if ((p2g_minb < 0 || p2g_minb == 1 || p2g_minb > 9) || (musl_minb < 0 || musl_minb == 1 || musl_minb > 7) ||
        update_ctas_per_sm < 0 || update_ctas_per_sm > 8)
        return MPM_ERR_BAD_ARG;
    c->tune.p2g_staged = p2g_minb == 0;
    c->tune.p2g_moments = p2g_minb >= 4 ? p2g_minb - 3 : 0;
    if (p2g_minb == 2 || p2g_minb == 3) c->tune.p2g_minb = p2g_minb;
    c->tune.musl_staged = musl_minb == 0 ? 1 : musl_minb == 4 ? 2 : 0;
    c->tune.musl_moments = musl_minb == 6 ? 1 : musl_minb == 7 ? 2 : 0;
    if (musl_minb == 2 || musl_minb == 3 || musl_minb == 5) c->tune.musl_minb = musl_minb;
    c->tune.update_ctas_per_sm = update_ctas_per_sm;
    return MPM_OK;
}

mpm_status mpm_gpu_get_tuning(mpm_ctx *c, int *p2g_minb, int *musl_minb, int *update_ctas_per_sm) {
    if (!c) return MPM_ERR_BAD_ARG;
    if (p2g_minb)
        *p2g_minb = c->tune.p2g_moments ? 3 + c->tune.p2g_moments : c->tune.p2g_staged ? 0 : c->tune.p2g_minb;
    if (musl_minb)
        *musl_minb = c->tune.musl_moments ? 5 + c->tune.musl_moments : c->tune.musl_staged == 2 ? 4 : c->tune.musl_staged ? 0 : c->tune.musl_minb;
    if (update_ctas_per_sm) *update_ctas_per_sm = c->tune.update_ctas_per_sm;
    return MPM_OK;
}

mpm_status mpm_gpu_enable_kernel_timing(mpm_ctx *c, int on) {
    if (!c) return MPM_ERR_BAD_ARG;
    c->timer.on = on != 0;
    return MPM_OK;
}

mpm_status mpm_gpu_kernel_times(mpm_ctx *c, int *count, const char **names, double *ms, int64_t *launches) {
    if (!c || !count) return MPM_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(c->stream));
    auto &t = c->timer;
    for (size_t i = 0; i < t.cls.size(); i++) {
        float e = 0.0f;
        cudaEventElapsedTime(&e, t.ev[2 * i], t.ev[2 * i + 1]);
        t.ms[t.cls[i]] += e;
        t.launches[t.cls[i]]++;
        cudaEventDestroy(t.ev[2 * i]);
        cudaEventDestroy(t.ev[2 * i + 1]);
    }
    t.ev.clear();
    t.cls.clear();
    int cap = *count, k = 0;
    for (int i = 0; i < NKCLASS && k < cap; i++) {
        if (names) names[k] = kClassNames[i];
        if (ms) ms[k] = t.ms[i];
        if (launches) launches[k] = t.launches[i];
        k++;
    }
    *count = k;
    for (int i = 0; i < NKCLASS; i++) {
        t.ms[i] = 0.0;
        t.launches[i] = 0;
    }
    return MPM_OK;
}


