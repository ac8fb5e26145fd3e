// fsi_abi.cu -- host implementation of the C-ABI declared in include/fsi_gpu.h.
//
// A block handle owns the device state of one LBMBlock (FluidDomain.f90:17-56):
// two distribution buffers (A/B, swapped every step), full-size den/uuu,
// half-way face copies, the immersed-boundary marker arrays and the IB window.
// Everything a time step needs stays resident in HBM; the host exchanges only
// marker data, the Lagrangian force and scalars.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <mutex>
#include <new>

#include <nvtx3/nvToolsExt.h>

#include "../../include/fsi_gpu.h"
#include "fsi_kernels.h"
#include "mlp_impl.cuh"

using namespace fsi;

namespace {
// One NVTX range per call of the entry points a time loop makes, named after
// the function, so that a profiler's timeline shows the host side of every
// step beside its kernels (a no-op when no profiler is attached).
struct CallRange {
    explicit CallRange(const char *name) { nvtxRangePushA(name); }
    ~CallRange() { nvtxRangePop(); }
    CallRange(const CallRange &) = delete;
    CallRange &operator=(const CallRange &) = delete;
};
}  // namespace
#define FSI_CALL_RANGE() CallRange fsi_call_range_(__func__)

static_assert(FSI_MLP_IN == MLP_IN && FSI_MLP_OUT == MLP_OUT, "perceptron shape");
static_assert(FSI_MLP_NPARAM == MLP_NP && FSI_MLP_NNORM == MLP_NNORM, "perceptron sizes");

// CTAs of the IB stage when it runs beside the bulk step: at least this many,
// about a sixth of the one-warp-per-marker grid (every IB CTA takes registers
// from the bulk step on its SM; measured on the 33x33-marker headline plate:
// 0.496 ms/step uncapped, 0.482 at 24 CTAs, 0.485 at 48, 0.488 at 80)
#ifndef FSI_IB_OVERLAP_CTAS
#define FSI_IB_OVERLAP_CTAS 24
#endif

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

}  // namespace

// the message of fsi_last_error for the host-side units (beam_host.cpp)
namespace fsi {
int host_fail(int code, const char *msg) {
    g_err = msg;
    return code;
}
}  // namespace fsi

namespace {

#define CK(call)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return fail(FSI_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

bool valid_code(int c) {
    switch (c) {
    case 0: case 1: case 101: case 102: case 103: case 104:
    case 201: case 202: case 203: case 204: case 301: case 302: return true;
    default: return false;
    }
}

size_t elem_size(int prec) {
    switch (prec) {
    case FSI_PREC_F64: case FSI_PREC_F64_FAST: return 8;
    case FSI_PREC_F32: return 4;
    default: return 2;
    }
}

// calculate_MRT_params (FluidDomain.f90:466-522): M from the Gram-Schmidt
// moment basis, M^-1 = M^T / diag(M M^T), M_COLLID = M^-1 S M, M_FORCE = I - M_COLLID/2.
void build_mrt(double omega, double *mc, double *mf) {
    const int Q_ = 19;
    double M[19][19], Mi[19][19], D[19], T[19][19];
    for (int k = 0; k < Q_; k++)
        for (int i = 0; i < Q_; i++) M[k][i] = (double)mrow_(k, i);
    for (int r = 0; r < Q_; r++) {
        double s = 0.0;
        for (int k = 0; k < Q_; k++) s += M[r][k] * M[r][k];
        D[r] = s;
    }
    for (int r = 0; r < Q_; r++)
        for (int c = 0; c < Q_; c++) Mi[r][c] = M[c][r] / D[c];
    const double s0 = 0.0, s1 = 1.19, s2 = 1.4, s4 = 1.2, s10 = 1.4, s16 = 1.98;  // ConstParams.f90:28
    const double S[19] = {s0, s1, s2, s0, s4, s0, s4, s0, s4, omega, s10, omega, s10, omega, omega, omega, s16, s16, s16};
    for (int r = 0; r < Q_; r++)
        for (int c = 0; c < Q_; c++) T[r][c] = Mi[r][c] * S[c];
    for (int r = 0; r < Q_; r++)
        for (int c = 0; c < Q_; c++) {
            double s = 0.0;
            for (int k = 0; k < Q_; k++) s += T[r][k] * M[k][c];
            mc[r + Q_ * c] = s;
            mf[r + Q_ * c] = (r == c ? 1.0 : 0.0) - 0.5 * s;
        }
}

// The moment form of a given M_COLLID/M_FORCE pair: S = M M_COLLID M^-1 must
// be diagonal with zeros on the conserved moments, and M_FORCE = I - M_COLLID/2.
void mrt_moment_form(MrtMats &m) {
    const int Q_ = 19;
    double M[19][19], D[19], T[19][19];
    for (int k = 0; k < Q_; k++) {
        D[k] = 0.0;
        for (int i = 0; i < Q_; i++) {
            M[k][i] = (double)mrow_(k, i);
            D[k] += M[k][i] * M[k][i];
        }
    }
    for (int k = 0; k < Q_; k++)
        for (int c = 0; c < Q_; c++) {
            double s = 0.0;
            for (int i = 0; i < Q_; i++) s += M[k][i] * m.mc[i + Q_ * c];
            T[k][c] = s;
        }
    bool ok = true;
    for (int k = 0; k < Q_ && ok; k++)
        for (int l = 0; l < Q_; l++) {
            double s = 0.0;
            for (int c = 0; c < Q_; c++) s += T[k][c] * M[l][c] / D[l];
            if (k == l) m.sd[k] = s / D[k];
            else if (std::fabs(s) > 1e-9) { ok = false; break; }
        }
    for (int k : {0, 3, 5, 7})
        if (std::fabs(m.sd[k]) > 1e-12) ok = false;
    for (int i = 0; i < Q_ * Q_ && ok; i++) {
        const double id = (i % Q_ == i / Q_) ? 1.0 : 0.0;
        if (std::fabs(m.mf[i] - (id - 0.5 * m.mc[i])) > 1e-12) ok = false;
    }
    m.diag = ok ? 1 : 0;
}

// the device status words (8 ints) followed by the IB residual (a double)
constexpr size_t STAT_BYTES = sizeof(int) * 8 + sizeof(double);
// streams the per-case form of a batch's bulk step fans out over
constexpr int BATCH_FAN = 16;

}  // namespace

struct fsi_block {
    fsi_block_desc d{};
    int X = 0, Y = 0, Z = 0;
    long long N = 0;
    double tau = 0, omega = 0, xmax = 0, ymax = 0, zmax = 0;
    double omega2 = 0;          // TRT antisymmetric rate
    double cles = 0;            // constant of the LES model (ConstParams.f90:40-45)
    double *tau_all = nullptr;  // per-cell relaxation time of the LES models (N), FP64 forms
    float *tauf = nullptr;      // the same in FP32 for the offset storage forms (current)
    float *tauf2 = nullptr;     // WALE, offset forms: the other buffer (the step reads one, writes the other)
    float *uf = nullptr;        // FP32 velocity field of WALE / Vreman, offset storage forms (3N)
    void *og = nullptr;         // WALE, fast forms: rotation-rate entries O12, O13, O23 (3N, arithmetic type)
    int periodic[3] = {0, 0, 0};
    MrtMats mm{};
    int prec = 0;               // storage form of every kernel but the bulk step
    bool dw = false;            // FSI_PREC_F64_DW: the bulk step in double-word arithmetic
    size_t esz = 8;
    void *fa = nullptr, *fb = nullptr;
    double *den = nullptr, *u = nullptr;
    double *stage = nullptr;  // FP64 staging for converted storage forms
    double *hw[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int hw_ready[6] = {0, 0, 0, 0, 0, 0};
    cudaStream_t st = nullptr;
    // ev_ibk: the IB stage's kernel done (the fluid step's window fix-up
    // waits for it); ev_ib: its force and status on the host as well
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_ib = nullptr, ev_ibk = nullptr;
    // the IB stage beside the bulk step (fsi_block_ib_step, FSI_IB_CLUSTER)
    int ib_mode = FSI_IB_AUTO;
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_fork = nullptr;
    double *h_ef = nullptr;  // pinned staging of the Lagrangian force (fsi_block_ib_step)
    int h_ef_cap = 0;
    void *d_out = nullptr;   // output packing scratch
    size_t out_cap = 0;
    // immersed boundary
    int nb = 0, Mtot = 0;
    std::vector<int> M, offs;
    int ibbc[6] = {0, 0, 0, 0, 0, 0};
    int *d_offs = nullptr, *d_err = nullptr;
    // d_vel and d_area point into the d_xyz allocation ([xyz 3M][vel 3M][area M]);
    // h_mk is its pinned mirror, so that one copy uploads the markers
    double *d_xyz = nullptr, *d_vel = nullptr, *d_area = nullptr, *d_eforce = nullptr, *d_fet = nullptr;
    double *h_mk = nullptr;
    double *d_tolm = nullptr, *d_tol = nullptr;
    int16_t *d_ei = nullptr;
    float *d_ew = nullptr;
    int *d_c64 = nullptr;       // fast forms: window cell and weight product of every stencil point
    double *d_w64 = nullptr;
    double *h_tol = nullptr;  // pinned
    int *h_err = nullptr;     // pinned
    // cooperative IB solve of the fast forms
    int coop_grid = 0;
    // 8 ints: IB flags, iterations, barrier count, generation; [4] the step
    // kernel's error word (bit 1: a bounded wait ran out)
    int *d_status = nullptr;
    int *h_stat = nullptr;  // pinned copy of d_status (STAT_BYTES: 8 status words, the IB residual)
    // the last cooperative IB stage ended cleanly and h_stat holds its status
    // (error word 0, the barrier counter in h_stat[2]): the next one starts
    // from that counter without clearing the status words
    bool ib_clean = false;
    double *d_res = nullptr, *d_tolacc = nullptr;
    int tolacc_cap = 0;
    // warm start: per-marker auxiliary inputs and logged features
    double *d_aux = nullptr;
    float *d_feat = nullptr;
    int warm_cap = 0;
    // IB window
    IbGeom geom{};
    long long Nw = 0, Nw_cap = 0;
    double *wden = nullptr, *wu = nullptr, *wforce = nullptr, *wu2 = nullptr, *dlt = nullptr;
    int *cnt = nullptr, *start = nullptr, *fillc = nullptr, *list = nullptr;
    long long list_cap = 0;
    bool win_valid = false;
    // fsi_block_ib_step_async: 1 the IB stage and step are queued, 2 (exact
    // form) the force waits in h_ef with pend_iters / pend_res
    int ib_pending = 0;
    int pend_iters = 0;
    double pend_res = 0.0;
    // captured graph of two steps (A->B, B->A)
    int kernel = FSI_KERNEL_AUTO;  // bulk step kernel of the offset forms
    cudaGraphExec_t gexec = nullptr;
    double g_vf[3] = {0, 0, 0};
    void *g_src = nullptr;
};

struct fsi_pair {
    fsi_block_t fa = nullptr, so = nullptr;
    PairGeom p{};
    int scheme = 1;
    double *buf[6][2] = {};
    double *buft[6][2] = {};
    double *scr_f = nullptr, *scr_t = nullptr;
    long long scr_cells = 0;
    int *d_err = nullptr;  // first out-of-range access of a face kernel: code, index lo, hi
};

// The warm-start perceptron: parameters, input/output statistics, Adam state
// and the training set, all resident on the device of its creation.
struct fsi_mlp {
    int dev = 0;
    cudaStream_t st = nullptr;
    float *P = nullptr, *nrm = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
    float *X = nullptr, *Y = nullptr;
    int *perm = nullptr, *hperm = nullptr;  // two epochs' sample orders, device and pinned host
    cudaEvent_t ev[2] = {nullptr, nullptr};  // each order slot's last use
    long long cap = 0;  // samples the training buffers hold
    int loss_cap = 0;
    int t = 0;          // Adam steps taken
    bool norm_set = false;
};

namespace {

bool is_fast(const fsi_block *h) { return h->prec != FSI_PREC_F64; }

// tau_all of a block for the refinement exchange
TauSrc tau_src(const fsi_block *h) { return TauSrc{h->tau, h->tau_all, h->tauf}; }

Vel make_vel(const fsi_block *h, double blktime) {
    Vel v{};
    v.kind = h->d.velocityKind;
    for (int i = 0; i < 3; i++) { v.vin[i] = h->d.uvwIn[i]; v.sr[i] = h->d.shearRateIn[i]; }
    // evaluate_oscillatory_velocity (FluidDomain.f90:1813-1824), uniform in space
    const double pi = 3.141592653589793;
    v.osc[0] = h->d.uvwIn[0] + h->d.shearRateIn[0] * cos(((2.0 * pi) * h->d.shearRateIn[1]) * blktime +
                                                         (h->d.shearRateIn[2] / 180.0) * pi);
    v.osc[1] = h->d.uvwIn[1];
    v.osc[2] = h->d.uvwIn[2];
    return v;
}

void face_dims(const fsi_block *h, int k, int &A, int &B) {
    int ax = k >> 1;
    A = (ax < 2) ? h->Z : h->Y;
    B = (ax == 0) ? h->Y : h->X;
}

// The arguments of face k's kernel on buffer f; false when face k has no
// kernel (periodic, fluid, a z face the step kernel wrote, or a half-way face
// on its first call). zdone[s]: the step kernel already wrote z face 4+s (the
// x/y faces then leave that plane alone, so that the z face stays the last
// writer there).
bool fill_bc(fsi_block *h, int k, void *f, double blktime, const int zdone[2], BcArgs &a) {
    const int zd0 = zdone ? zdone[0] : 0, zd1 = zdone ? zdone[1] : 0;
    int code = h->d.bndConds[k];
    if (code == BC_PERIODIC || code == BC_FLUID || code == BC_FLUID_FATHER) return false;
    if ((k == 4 && zd0) || (k == 5 && zd1)) return false;
    if (code == BC_WALL_HW || code == BC_MWALL_HW) {
        // allocate-on-first-call semantics, FluidDomain.f90:660-662
        if (!h->hw_ready[k]) { h->hw_ready[k] = 1; return false; }
    }
    a = BcArgs{};
    a.f = f;
    a.X = h->X; a.Y = h->Y; a.Z = h->Z; a.N = h->N;
    a.face = k; a.code = code;
    a.dh = h->d.dh; a.xmin = h->d.xmin; a.ymin = h->d.ymin; a.zmin = h->d.zmin;
    a.xmax = h->xmax; a.ymax = h->ymax; a.zmax = h->zmax;
    a.denIn = h->d.denIn;
    a.vel = make_vel(h, blktime);
    a.hw = h->hw[k];
    a.den = h->den;
    a.u = h->u;
    a.zlo = zd0 ? 1 : 0;
    a.zhi = h->Z - 1 - (zd1 ? 1 : 0);
    // offset forms, code 101: a face velocity uniform over the face (no shear
    // along the face's own coordinates) gives one set of face populations
    const bool off = h->prec == FSI_PREC_F32 || h->prec == FSI_PREC_F16 || h->prec == FSI_PREC_BF16;
    const int ax = k >> 1;
    const Vel &v = a.vel;
    const bool uniform = v.kind == 2 || (ax == 0 ? (v.sr[1] == 0.0 && v.sr[2] == 0.0)
                                                 : ax == 1 ? (v.sr[0] == 0.0 && v.sr[2] == 0.0)
                                                           : (v.sr[0] == 0.0 && v.sr[1] == 0.0));
    if (off && code == BC_EQ && uniform) {
        // evaluate_velocity at the face (FluidDomain.f90:1791-1824)
        const double xc = ax == 0 ? ((k & 1) ? h->xmax : h->d.xmin) : h->d.xmin;
        const double yc = ax == 1 ? ((k & 1) ? h->ymax : h->d.ymin) : h->d.ymin;
        const double zc = ax == 2 ? ((k & 1) ? h->zmax : h->d.zmin) : h->d.zmin;
        double u[3];
        if (v.kind == 2) {
            u[0] = v.osc[0]; u[1] = v.osc[1]; u[2] = v.osc[2];
        } else {
            u[0] = ((v.vin[0] + 0.0 * v.sr[0]) + yc * v.sr[1]) + zc * v.sr[2];
            u[1] = ((v.vin[1] + xc * v.sr[0]) + 0.0 * v.sr[1]) + zc * v.sr[2];
            u[2] = ((v.vin[2] + xc * v.sr[0]) + yc * v.sr[1]) + 0.0 * v.sr[2];
        }
        // the offset equilibrium (calculate_distribution_funcion,
        // FluidDomain.f90:1827-1834, minus the weight), as for the z faces
        const double rho = h->d.denIn, usq = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2];
        for (int q = 0; q < 19; q++) {
            const double eu = (u[0] * ex_(q) + u[1] * ey_(q)) + u[2] * ez_(q);
            a.gq[q] = (float)(wt_(q) * (rho - 1.0) + (wt_(q) * rho) * ((3.0 + 4.5 * eu) * eu - 1.5 * usq));
        }
        a.uni = 1;
    }
    return true;
}

int apply_bcs(fsi_block *h, void *f, double blktime, const int zdone[2] = nullptr) {
    const bool off = h->prec == FSI_PREC_F32 || h->prec == FSI_PREC_F16 || h->prec == FSI_PREC_BF16;
    for (int ax = 0; ax < 3; ax++) {
        BcArgs a[2];
        bool on[2];
        for (int s = 0; s < 2; s++) on[s] = fill_bc(h, 2 * ax + s, f, blktime, zdone, a[s]);
        // the two faces of an axis in one launch when each reads and writes
        // only its own three layers and the axis keeps them apart
        const int D = ax == 0 ? h->X : (ax == 1 ? h->Y : h->Z);
        if (off && on[0] && on[1] && D >= 6) {
            cudaError_t e = launch_bc_pair_fast(a[0], a[1], h->prec, h->st);
            if (e != cudaSuccess) return fail(FSI_E_CUDA, "boundary kernel: %s", cudaGetErrorString(e));
            continue;
        }
        for (int s = 0; s < 2; s++) {
            if (!on[s]) continue;
            cudaError_t e = is_fast(h) ? launch_bc_fast(a[s], h->prec, h->st) : launch_bc_f64(a[s], h->st);
            if (e != cudaSuccess) return fail(FSI_E_CUDA, "boundary kernel: %s", cudaGetErrorString(e));
        }
    }
    return FSI_OK;
}

// the arguments of one fluid step of h (fa -> fb)
void fill_step(fsi_block *h, const double vf[3], double blktime, bool use_window, StepArgs &a) {
    a = StepArgs{};
    a.src = h->fa;
    a.dst = h->fb;
    a.X = h->X; a.Y = h->Y; a.Z = h->Z; a.N = h->N;
    a.dh = h->d.dh;
    a.omega = h->omega;
    for (int i = 0; i < 3; i++) a.vf[i] = vf[i];
    if (use_window && h->win_valid) {
        a.win.x0 = h->geom.wx0; a.win.x1 = h->geom.wx1;
        a.win.y0 = h->geom.wy0; a.win.y1 = h->geom.wy1;
        a.win.z0 = h->geom.wz0; a.win.z1 = h->geom.wz1;
        a.win.WY = h->geom.WY; a.win.WZ = h->geom.WZ;
        a.win.n = h->Nw;
        a.win.den = h->wden; a.win.u = h->wu; a.win.force = h->wforce;
    } else {
        a.win.x0 = 0; a.win.x1 = -1; a.win.y0 = 0; a.win.y1 = -1; a.win.z0 = 0; a.win.z1 = -1;
    }
    for (int k = 0; k < 6; k++) {
        int code = h->d.bndConds[k];
        a.hw[k] = (code == BC_WALL_HW || code == BC_MWALL_HW) ? h->hw[k] : nullptr;
        a.l2[k] = (code == BC_NEQ) ? 1 : 0;
    }
    a.den = h->den;
    a.u = h->u;
    a.kerr = h->d_status + 4;
    a.variant = h->kernel;
    a.omega2 = h->omega2;
    a.tau = h->tau;
    a.nu = h->d.nu;
    a.cles = h->cles;
    a.tau_all = h->tau_all;
    // WALE in the offset forms reads the current tau_all and writes the other
    // buffer (swapped with the distributions after the step)
    a.tauf = h->tauf2 ? h->tauf2 : h->tauf;
    a.tauf_prev = h->tauf;
    a.uf = h->uf;
    a.og = h->og;
    // z faces of code 101 with a face velocity uniform over the face: the
    // paired kernels write their equilibrium while streaming
    if (is_fast(h) && step_fast_paired(a, &h->mm, h->prec, h->d.iCollidModel)) {
        const Vel v = make_vel(h, blktime);
        const bool uniform = v.kind == 2 || (v.sr[0] == 0.0 && v.sr[1] == 0.0);
        for (int s = 0; s < 2; s++) {
            if (h->d.bndConds[4 + s] != BC_EQ || !uniform) continue;
            // evaluate_velocity at the face (FluidDomain.f90:1791-1824)
            const double zc = s ? h->zmax : h->d.zmin;
            double u[3];
            if (v.kind == 2) {
                u[0] = v.osc[0]; u[1] = v.osc[1]; u[2] = v.osc[2];
            } else {
                u[0] = ((v.vin[0] + 0.0 * v.sr[0]) + h->d.ymin * v.sr[1]) + zc * v.sr[2];
                u[1] = ((v.vin[1] + h->d.xmin * v.sr[0]) + 0.0 * v.sr[1]) + zc * v.sr[2];
                u[2] = ((v.vin[2] + h->d.xmin * v.sr[0]) + h->d.ymin * v.sr[1]) + 0.0 * v.sr[2];
            }
            // offset equilibrium of the face (calculate_distribution_funcion,
            // FluidDomain.f90:1827-1834, minus the weight)
            const double rho = h->d.denIn, usq = (u[0] * u[0] + u[1] * u[1]) + u[2] * u[2];
            for (int q = 0; q < 19; q++) {
                const double eu = (u[0] * ex_(q) + u[1] * ey_(q)) + u[2] * ez_(q);
                a.zg[s][q] = (float)(wt_(q) * (rho - 1.0) + (wt_(q) * rho) * ((3.0 + 4.5 * eu) * eu - 1.5 * usq));
            }
            a.zeq[s] = 1;
        }
    }
}

int enqueue_step(fsi_block *h, const double vf[3], double blktime, bool use_window, cudaEvent_t join = nullptr) {
    StepArgs a;
    fill_step(h, vf, blktime, use_window, a);
    a.join = (void *)join;
    cudaError_t e = cudaSuccess;
    // only the paired kernels defer their IB-window work behind the join
    // event; every other step, and the velocity pass of the gradient
    // models, waits for the IB stage before it starts
    if (join && (grad_model(h->d.iCollidModel) || !(is_fast(h) && step_fast_paired(a, &h->mm, h->prec,
                                                                                    h->d.iCollidModel)))) {
        e = cudaStreamWaitEvent(h->st, join, 0);
        a.join = nullptr;
    }
    if (e == cudaSuccess && grad_model(h->d.iCollidModel))
        e = is_fast(h) ? launch_step_macro_fast(a, h->prec, h->st) : launch_step_macro_f64(a, h->st);
    if (e == cudaSuccess)
        e = is_fast(h) ? launch_step_fast(a, &h->mm, h->dw ? FSI_PREC_F64_DW : h->prec, h->d.iCollidModel, h->st)
                       : launch_step_f64_exact(a, &h->mm, h->d.iCollidModel, h->st);
    if (e != cudaSuccess) return fail(FSI_E_CUDA, "step kernel: %s", cudaGetErrorString(e));
    int rc = apply_bcs(h, h->fb, blktime, a.zeq);
    if (rc) return rc;
    std::swap(h->fa, h->fb);
    if (h->tauf2) std::swap(h->tauf, h->tauf2);
    return FSI_OK;
}

// the step kernel's error word, read after the stream has drained
int check_kerr(fsi_block *h) {
    CK(cudaMemcpyAsync(h->h_stat + 4, h->d_status + 4, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (h->h_stat[4]) return fail(FSI_E_TIMEOUT, "step kernel: a bounded wait ran out");
    return FSI_OK;
}

void free_block(fsi_block *h) {
    if (!h) return;
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    void *ptrs[] = {h->fa, h->fb, h->den, h->u, h->stage, h->d_offs, h->d_err, h->d_xyz,
                    h->d_eforce, h->d_fet, h->d_tolm, h->d_tol, h->d_ei, h->d_ew, h->wden, h->wu, h->wforce,
                    h->wu2, h->dlt, h->cnt, h->start, h->fillc, h->list, h->d_status, h->d_tolacc, h->d_aux,
                    h->d_feat, h->d_out, h->tau_all, h->tauf, h->uf, h->og, h->tauf2, h->d_c64, h->d_w64};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int k = 0; k < 6; k++)
        if (h->hw[k]) cudaFree(h->hw[k]);
    if (h->h_tol) cudaFreeHost(h->h_tol);
    if (h->h_err) cudaFreeHost(h->h_err);
    if (h->h_stat) cudaFreeHost(h->h_stat);
    if (h->h_mk) cudaFreeHost(h->h_mk);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->ev_ib) cudaEventDestroy(h->ev_ib);
    if (h->ev_ibk) cudaEventDestroy(h->ev_ibk);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->st2) cudaStreamDestroy(h->st2);
    if (h->h_ef) cudaFreeHost(h->h_ef);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
}

}  // namespace

extern "C" {

int fsi_last_error(char *buf, int len) {
    int n = (int)g_err.size();
    if (buf && len > 0) {
        int m = std::min(n, len - 1);
        memcpy(buf, g_err.data(), m);
        buf[m] = 0;
    }
    return n;
}

int fsi_device_info(int *sm_count, int *cc_major, int *cc_minor) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    cudaDeviceProp p;
    CK(cudaGetDeviceProperties(&p, dev));
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    return FSI_OK;
}

int fsi_block_create(fsi_block_t *out, const fsi_block_desc *d) {
    if (!out || !d) return fail(FSI_E_ARG, "null argument");
    *out = nullptr;
    if (d->xDim < 3 || d->yDim < 3 || d->zDim < 3) return fail(FSI_E_ARG, "block dimensions must be >= 3");
    // FluidDomain.f90:88-91: marker stencil indices are int16
    if (d->xDim > 32767 || d->yDim > 32767 || d->zDim > 32767)
        return fail(FSI_E_ARG, "Grid number exceeds 32767, please try to reduced the grid size.");
    if (!(d->dh > 0.0)) return fail(FSI_E_ARG, "dh must be positive");
    if (d->iCollidModel == 12)
        return fail(FSI_E_ARG, "iCollidModel 12 (RBGK) is not supported: the reference's branch relaxes with an "
                               "uninitialised rate (FluidDomain.f90:1240-1243)");
    if (d->iCollidModel == 13)
        return fail(FSI_E_ARG, "iCollidModel 13 (ELBM) is not supported: the reference's branch sums an "
                               "uninitialised array x3 (FluidDomain.f90:1296-1301)");
    {
        const int m = d->iCollidModel;
        if (m != CM_SRT && m != CM_TRT && m != CM_MRT && !les_model(m))
            return fail(FSI_E_ARG, "iCollidModel %d not supported (1 SRT, 2 TRT, 3 MRT, 11 Smagorinsky, 14 WALE, "
                                   "15 Vreman)", m);
    }
    if (d->precision < FSI_PREC_F64 || d->precision > FSI_PREC_F64_DW) return fail(FSI_E_ARG, "unknown precision");
    if (d->precision == FSI_PREC_F64_DW && d->iCollidModel != CM_SRT && d->iCollidModel != CM_MRT)
        return fail(FSI_E_ARG, "the double-word form computes SRT and MRT collisions only (iCollidModel %d)",
                    d->iCollidModel);
    if (d->velocityKind != 0 && d->velocityKind != 2)
        return fail(FSI_E_ARG, "velocityKind %d not supported (0 shear, 2 oscillatory)", d->velocityKind);
    for (int k = 0; k < 6; k++)
        if (!valid_code(d->bndConds[k])) return fail(FSI_E_BC, "face %d has no such boundary condition %d", k, d->bndConds[k]);
    // check_periodic_boundary_ (FluidDomain.f90:110-125)
    for (int i = 0; i < 3; i++) {
        int a = d->bndConds[2 * i], b = d->bndConds[2 * i + 1];
        if ((a == BC_PERIODIC || b == BC_PERIODIC) && a != b)
            return fail(FSI_E_BC, "Stop! Periodic boundaries must apper in pairs: %d %d", a, b);
    }
    fsi_block *h = new (std::nothrow) fsi_block();
    if (!h) return fail(FSI_E_ARG, "out of host memory");
    h->d = *d;
    h->d.m_collid = nullptr;
    h->d.m_force = nullptr;
    h->X = d->xDim; h->Y = d->yDim; h->Z = d->zDim;
    h->N = (long long)h->X * h->Y * h->Z;
    for (int i = 0; i < 3; i++) h->periodic[i] = (d->bndConds[2 * i] == BC_PERIODIC) ? 1 : 0;
    // FluidDomain.f90:94-105
    h->xmax = d->xmin + d->dh * (double)(h->X - 1);
    h->ymax = d->ymin + d->dh * (double)(h->Y - 1);
    h->zmax = d->zmin + d->dh * (double)(h->Z - 1);
    if (h->periodic[0]) h->xmax = h->xmax + d->dh;
    if (h->periodic[1]) h->ymax = h->ymax + d->dh;
    if (h->periodic[2]) h->zmax = h->zmax + d->dh;
    // calculate_SRT_params, FluidDomain.f90:450-456
    h->tau = d->nu / (d->dh * (1.0 / 3.0)) + 0.5;
    h->omega = 1.0 / h->tau;
    // calculate_TRT_params, FluidDomain.f90:458-464
    if (d->iCollidModel == CM_TRT) {
        const double tmp = (d->params[0] * 4.0 - 1.0) * h->omega + 2.0;
        h->omega2 = (2.0 * (2.0 - h->omega)) / tmp;
        if (!std::isfinite(h->omega2)) {
            delete h;
            return fail(FSI_E_ARG, "TRT: Lambda %g gives no finite Omega2", d->params[0]);
        }
    }
    // CsmagConst, CWALEConst, CvremConst (ConstParams.f90:40-45), each
    // product rounded in turn
    if (d->iCollidModel == CM_SMAG) h->cles = ((2.0 * 0.17) * 0.17) * std::sqrt(2.0) * 9.0;
    else if (d->iCollidModel == CM_WALE) h->cles = 0.5 * 0.5;
    else if (d->iCollidModel == CM_VREM) h->cles = (2.5 * 0.17) * 0.17;
    if (d->m_collid && d->m_force) {
        memcpy(h->mm.mc, d->m_collid, sizeof(double) * 361);
        memcpy(h->mm.mf, d->m_force, sizeof(double) * 361);
    } else {
        build_mrt(h->omega, h->mm.mc, h->mm.mf);
    }
    mrt_moment_form(h->mm);
    if (d->precision == FSI_PREC_F64_DW && d->iCollidModel == CM_MRT && !h->mm.diag) {
        delete h;
        return fail(FSI_E_ARG, "the double-word form needs MRT matrices of the moment form M^-1 S M");
    }
    // the double-word form stores FP64 like FSI_PREC_F64_FAST and shares its
    // kernels except the bulk step
    h->dw = d->precision == FSI_PREC_F64_DW;
    h->prec = h->dw ? FSI_PREC_F64_FAST : d->precision;
    h->esz = elem_size(h->prec);
    size_t fbytes = h->esz * 19 * (size_t)h->N;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    chk(cudaEventCreate(&h->ev0));
    chk(cudaEventCreate(&h->ev1));
    chk(cudaEventCreateWithFlags(&h->ev_ib, cudaEventDisableTiming));
    chk(cudaEventCreateWithFlags(&h->ev_ibk, cudaEventDisableTiming));
    chk(cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    {
        // the IB stage's stream is served first when SMs free up
        int lo = 0, hi = 0;
        chk(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        chk(cudaStreamCreateWithPriority(&h->st2, cudaStreamNonBlocking, hi));
    }
    chk(cudaMalloc(&h->fa, fbytes));
    chk(cudaMalloc(&h->fb, fbytes));
    chk(cudaMalloc((void **)&h->den, sizeof(double) * h->N));
    chk(cudaMalloc((void **)&h->u, sizeof(double) * 3 * h->N));
    {
        const bool off = h->prec == FSI_PREC_F32 || h->prec == FSI_PREC_F16 || h->prec == FSI_PREC_BF16;
        if (les_model(d->iCollidModel) && off) {
            chk(cudaMalloc((void **)&h->tauf, sizeof(float) * h->N));
            if (e == cudaSuccess) chk(launch_fill_f32(h->tauf, h->N, (float)h->tau, h->st));
            if (d->iCollidModel == CM_WALE) {
                chk(cudaMalloc((void **)&h->tauf2, sizeof(float) * h->N));
                if (e == cudaSuccess) chk(launch_fill_f32(h->tauf2, h->N, (float)h->tau, h->st));
            }
        } else if (les_model(d->iCollidModel)) {
            chk(cudaMalloc((void **)&h->tau_all, sizeof(double) * h->N));
            if (e == cudaSuccess) chk(launch_fill_f64(h->tau_all, h->N, h->tau, h->st));
        }
        if (grad_model(d->iCollidModel) && off) chk(cudaMalloc((void **)&h->uf, sizeof(float) * 3 * h->N));
        if (d->iCollidModel == CM_WALE && h->prec != FSI_PREC_F64)
            chk(cudaMalloc(&h->og, (off ? sizeof(float) : sizeof(double)) * 3 * h->N));
    }
    if (h->prec != FSI_PREC_F64 && h->prec != FSI_PREC_F64_FAST)
        chk(cudaMalloc((void **)&h->stage, sizeof(double) * 19 * (size_t)h->N));
    for (int k = 0; k < 6; k++) {
        int code = d->bndConds[k];
        if (code == BC_WALL_HW || code == BC_MWALL_HW) {
            int A, B;
            face_dims(h, k, A, B);
            chk(cudaMalloc((void **)&h->hw[k], sizeof(double) * 19 * (size_t)A * B));
            if (e == cudaSuccess) chk(cudaMemsetAsync(h->hw[k], 0, sizeof(double) * 19 * (size_t)A * B, h->st));
        }
    }
    chk(cudaHostAlloc((void **)&h->h_tol, sizeof(double) * 64, cudaHostAllocDefault));
    chk(cudaHostAlloc((void **)&h->h_err, sizeof(int), cudaHostAllocDefault));
    chk(cudaMalloc((void **)&h->d_err, sizeof(int)));
    // the status words and the IB residual in one allocation (and one pinned
    // mirror), so that one copy brings both back
    chk(cudaMalloc((void **)&h->d_status, STAT_BYTES));
    if (h->d_status) h->d_res = (double *)(h->d_status + 8);
    chk(cudaHostAlloc((void **)&h->h_stat, STAT_BYTES, cudaHostAllocDefault));
    // every device operation of a block goes to its own (non-blocking)
    // stream: work on the legacy default stream would not be ordered with it
    if (e == cudaSuccess) chk(cudaMemsetAsync(h->den, 0, sizeof(double) * h->N, h->st));
    if (e == cudaSuccess) chk(cudaMemsetAsync(h->u, 0, sizeof(double) * 3 * h->N, h->st));
    if (e == cudaSuccess) chk(cudaMemsetAsync(h->fa, 0, fbytes, h->st));
    if (e == cudaSuccess) chk(cudaMemsetAsync(h->fb, 0, fbytes, h->st));
    if (e == cudaSuccess) chk(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->st));
    if (e == cudaSuccess) chk(cudaMemsetAsync(h->d_status, 0, sizeof(int) * 8, h->st));
    if (e == cudaSuccess) chk(cudaStreamSynchronize(h->st));
    if (e != cudaSuccess) {
        free_block(h);
        return fail(FSI_E_CUDA, "block allocation: %s", cudaGetErrorString(e));
    }
    *out = h;
    return FSI_OK;
}

int fsi_block_destroy(fsi_block_t h) {
    if (!h) return FSI_OK;
    // a queued IB step's copies run on the second stream
    cudaStreamSynchronize(h->st2);
    cudaStreamSynchronize(h->st);
    free_block(h);
    return FSI_OK;
}

int fsi_block_get_params(fsi_block_t h, double *tau, double *omega, double *m_collid, double *m_force) {
    if (!h) return fail(FSI_E_ARG, "null handle");
    if (tau) *tau = h->tau;
    if (omega) *omega = h->omega;
    if (m_collid) memcpy(m_collid, h->mm.mc, sizeof(double) * 361);
    if (m_force) memcpy(m_force, h->mm.mf, sizeof(double) * 361);
    return FSI_OK;
}

int fsi_block_get_omega2(fsi_block_t h, double *omega2) {
    if (!h || !omega2) return fail(FSI_E_ARG, "null argument");
    *omega2 = h->omega2;
    return FSI_OK;
}

int fsi_block_get_tau_all(fsi_block_t h, double *tau_all) {
    if (!h || !tau_all) return fail(FSI_E_ARG, "null argument");
    if (h->tauf) {
        std::vector<float> t((size_t)h->N);
        CK(cudaMemcpyAsync(t.data(), h->tauf, sizeof(float) * h->N, cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        for (long long i = 0; i < h->N; i++) tau_all[i] = (double)t[(size_t)i];
        return FSI_OK;
    }
    if (!h->tau_all) {
        for (long long i = 0; i < h->N; i++) tau_all[i] = h->tau;
        return FSI_OK;
    }
    CK(cudaMemcpyAsync(tau_all, h->tau_all, sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return FSI_OK;
}

int fsi_block_upload_f(fsi_block_t h, const double *fIn) {
    FSI_CALL_RANGE();
    if (!h || !fIn) return fail(FSI_E_ARG, "null argument");
    size_t n = 19 * (size_t)h->N;
    if (h->esz == 8) {
        CK(cudaMemcpyAsync(h->fa, fIn, n * 8, cudaMemcpyHostToDevice, h->st));
    } else {
        CK(cudaMemcpyAsync(h->stage, fIn, n * 8, cudaMemcpyHostToDevice, h->st));
        CK(launch_convert_to_store(h->stage, h->fa, h->N, h->prec, h->st));
    }
    CK(cudaStreamSynchronize(h->st));
    return FSI_OK;
}

int fsi_block_download_f(fsi_block_t h, double *fIn) {
    FSI_CALL_RANGE();
    if (!h || !fIn) return fail(FSI_E_ARG, "null argument");
    size_t n = 19 * (size_t)h->N;
    if (h->esz == 8) {
        CK(cudaMemcpyAsync(fIn, h->fa, n * 8, cudaMemcpyDeviceToHost, h->st));
    } else {
        CK(launch_convert_from_store(h->fa, h->stage, h->N, h->prec, h->st));
        CK(cudaMemcpyAsync(fIn, h->stage, n * 8, cudaMemcpyDeviceToHost, h->st));
    }
    return check_kerr(h);
}

// ---------------------------------------------------------------- restart

int fsi_continue_write(const char *path, const fsi_block_t *blocks, int n, int step, double time) {
    FSI_CALL_RANGE();
    if (!path || !blocks || n <= 0) return fail(FSI_E_ARG, "invalid argument");
    for (int i = 0; i < n; i++)
        if (!blocks[i]) return fail(FSI_E_ARG, "null block %d", i);
    FILE *fp = fopen(path, "wb");
    if (!fp) return fail(FSI_E_ARG, "cannot open %s for writing", path);
    bool ok = true;
    const int32_t head[2] = {(int32_t)n, (int32_t)step};
    ok = ok && fwrite(head, sizeof(int32_t), 2, fp) == 2;
    ok = ok && fwrite(&time, sizeof(double), 1, fp) == 1;
    std::vector<double> f;
    int rc = FSI_OK;
    for (int i = 0; i < n && ok && rc == FSI_OK; i++) {
        fsi_block *h = blocks[i];
        const double g[4] = {h->d.xmin, h->d.ymin, h->d.zmin, h->d.dh};
        const int32_t dims[3] = {(int32_t)h->X, (int32_t)h->Y, (int32_t)h->Z};
        f.resize(19 * (size_t)h->N);
        rc = fsi_block_download_f(h, f.data());
        if (rc) break;
        ok = ok && fwrite(g, sizeof(double), 4, fp) == 4;
        ok = ok && fwrite(dims, sizeof(int32_t), 3, fp) == 3;
        ok = ok && fwrite(f.data(), sizeof(double), f.size(), fp) == f.size();
    }
    if (fclose(fp) != 0) ok = false;
    if (rc) return rc;
    if (!ok) return fail(FSI_E_ARG, "short write to %s", path);
    return FSI_OK;
}

int fsi_continue_read(const char *path, const fsi_block_t *blocks, int n, int *step, double *time) {
    FSI_CALL_RANGE();
    if (!path || !blocks || n <= 0) return fail(FSI_E_ARG, "invalid argument");
    for (int i = 0; i < n; i++)
        if (!blocks[i]) return fail(FSI_E_ARG, "null block %d", i);
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(FSI_E_ARG, "cannot open %s", path);
    fseek(fp, 0, SEEK_END);
    const long long fsize = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    int32_t head[2];
    double t0 = 0.0;
    if (fread(head, sizeof(int32_t), 2, fp) != 2 || fread(&t0, sizeof(double), 1, fp) != 1 || head[0] <= 0) {
        fclose(fp);
        return fail(FSI_E_ARG, "%s: not a continue file", path);
    }
    const int nold = head[0];
    long long pos = 16;
    std::vector<RegridSrc> src(nold);
    std::vector<double *> dev(nold, nullptr);
    std::vector<double> host;
    auto cleanup = [&]() {
        for (double *p : dev)
            if (p) cudaFree(p);
    };
    cudaStream_t st = blocks[0]->st;
    for (int k = 0; k < nold; k++) {
        double g[4];
        int32_t dims[3];
        if (fread(g, sizeof(double), 4, fp) != 4 || fread(dims, sizeof(int32_t), 3, fp) != 3 || dims[0] < 2 ||
            dims[1] < 2 || dims[2] < 2 || !(g[3] > 0.0)) {
            fclose(fp);
            cleanup();
            return fail(FSI_E_ARG, "%s: bad header of block %d", path, k);
        }
        pos += 44;
        const long long cells = (long long)dims[0] * dims[1] * dims[2];
        if (pos + 19 * 8 * cells > fsize) {
            fclose(fp);
            cleanup();
            return fail(FSI_E_ARG, "%s: block %d is truncated", path, k);
        }
        host.resize(19 * (size_t)cells);
        if (fread(host.data(), sizeof(double), host.size(), fp) != host.size()) {
            fclose(fp);
            cleanup();
            return fail(FSI_E_ARG, "%s: short read in block %d", path, k);
        }
        pos += 19 * 8 * cells;
        RegridSrc &r = src[k];
        r.xmin = g[0]; r.ymin = g[1]; r.zmin = g[2]; r.dh = g[3];
        r.X = dims[0]; r.Y = dims[1]; r.Z = dims[2];
        // coor_max, FluidDomain.f90:165-169
        r.xmx = r.xmin + (double)(r.X - 1) * r.dh;
        r.ymx = r.ymin + (double)(r.Y - 1) * r.dh;
        r.zmx = r.zmin + (double)(r.Z - 1) * r.dh;
        cudaError_t e = cudaMalloc((void **)&dev[k], sizeof(double) * host.size());
        if (e == cudaSuccess) e = cudaMemcpyAsync(dev[k], host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            fclose(fp);
            cleanup();
            return fail(FSI_E_CUDA, "continue upload: %s", cudaGetErrorString(e));
        }
        r.f = dev[k];
    }
    fclose(fp);
    // the search order: the exchange sort of FluidDomain.f90:151-163, which
    // compares dh at the original positions while it permutes the indices
    std::vector<int> order(nold);
    for (int i = 0; i < nold; i++) order[i] = i;
    for (int i = 0; i < nold - 1; i++)
        for (int j = i + 1; j < nold; j++)
            if (src[i].dh > src[j].dh) std::swap(order[i], order[j]);
    std::vector<RegridSrc> sorted(nold);
    for (int i = 0; i < nold; i++) sorted[i] = src[order[i]];
    RegridSrc *d_src = nullptr;
    int *d_err = nullptr;
    cudaError_t e = cudaMalloc((void **)&d_src, sizeof(RegridSrc) * nold);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_err, sizeof(int) * 4);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_src, sorted.data(), sizeof(RegridSrc) * nold, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(int) * 4, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    int herr[3] = {0, 0, 0};
    for (int i = 0; i < n && e == cudaSuccess; i++) {
        fsi_block *h = blocks[i];
        double *dst = (h->esz == 8) ? (double *)h->fa : h->stage;
        if (h->esz != 8) e = launch_convert_from_store(h->fa, h->stage, h->N, h->prec, h->st);
        if (e == cudaSuccess)
            e = launch_regrid_f64(dst, h->X, h->Y, h->Z, h->d.dh, h->d.xmin, h->d.ymin, h->d.zmin, d_src, nold, d_err,
                                  h->st);
        if (e == cudaSuccess && h->esz != 8) e = launch_convert_to_store(h->stage, h->fa, h->N, h->prec, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(herr, d_err, sizeof(int) * 3, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (d_src) cudaFree(d_src);
    if (d_err) cudaFree(d_err);
    cleanup();
    if (e != cudaSuccess) return fail(FSI_E_CUDA, "continue re-grid: %s", cudaGetErrorString(e));
    if (herr[0]) return fail(FSI_E_RANGE, "continue re-grid: stencil outside a file block at cell %lld",
                             (long long)(unsigned)herr[1] | ((long long)herr[2] << 32));
    if (step) *step = head[1];
    if (time) *time = t0;
    return FSI_OK;
}

// ---------------------------------------------------------------- outputs

namespace {
// den/u of the current state into the block's full-size arrays
int macro_device(fsi_block *h, const double vf[3]) {
    double z3[3] = {0, 0, 0};
    const double *v = vf ? vf : z3;
    if (h->prec == FSI_PREC_F64) CK(launch_macro_f64((const double *)h->fa, h->den, h->u, h->X, h->Y, h->Z, h->d.dh, v, h->st));
    else CK(launch_macro_fast(h->fa, h->prec, h->den, h->u, h->X, h->Y, h->Z, h->d.dh, v, h->st));
    return FSI_OK;
}

int out_scratch(fsi_block *h, size_t bytes) {
    if (bytes <= h->out_cap) return FSI_OK;
    CK(cudaStreamSynchronize(h->st));
    if (h->d_out) cudaFree(h->d_out);
    h->d_out = nullptr;
    h->out_cap = 0;
    CK(cudaMalloc(&h->d_out, bytes));
    h->out_cap = bytes;
    return FSI_OK;
}
}  // namespace

int fsi_block_pack_flow(fsi_block_t h, const double vf[3], double denIn, double Uref, int offset, float *out) {
    FSI_CALL_RANGE();
    if (!h || !out) return fail(FSI_E_ARG, "null argument");
    if (!(Uref != 0.0)) return fail(FSI_E_ARG, "Uref must be nonzero");
    if (offset < 0 || 2 * offset >= h->X || 2 * offset >= h->Y || 2 * offset >= h->Z)
        return fail(FSI_E_ARG, "offset %d leaves no output cells", offset);
    const size_t n = (size_t)(h->X - 2 * offset) * (h->Y - 2 * offset) * (h->Z - 2 * offset);
    if (int rc = macro_device(h, vf)) return rc;
    if (int rc = out_scratch(h, sizeof(float) * 4 * n)) return rc;
    CK(launch_pack_flow(h->den, h->u, h->X, h->Y, h->Z, offset, denIn, Uref, (float *)h->d_out, h->st));
    CK(cudaMemcpyAsync(out, h->d_out, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, h->st));
    return check_kerr(h);
}

int fsi_block_flux(fsi_block_t h, const double vf[3], double denIn, double Uref, double flux[3]) {
    FSI_CALL_RANGE();
    if (!h || !flux) return fail(FSI_E_ARG, "null argument");
    if (int rc = macro_device(h, vf)) return rc;
    if (int rc = out_scratch(h, sizeof(double) * 3)) return rc;
    CK(launch_flux(h->den, h->u, h->X, h->Y, h->Z, h->d.dh, (double *)h->d_out, h->st));
    double raw[3];
    CK(cudaMemcpyAsync(raw, h->d_out, sizeof(double) * 3, cudaMemcpyDeviceToHost, h->st));
    if (int rc = check_kerr(h)) return rc;
    const double Yref = h->ymax - h->d.ymin, Zref = h->zmax - h->d.zmin;
    for (int k = 0; k < 3; k++) flux[k] = raw[k] / (((denIn * Uref) * Zref) * Yref);
    return FSI_OK;
}

int fsi_block_probes(fsi_block_t h, const double vf[3], int n, const double *xyz, double Uref, double *uvw) {
    FSI_CALL_RANGE();
    if (!h || n < 0 || (n > 0 && (!xyz || !uvw))) return fail(FSI_E_ARG, "invalid argument");
    if (n == 0) return FSI_OK;
    const double xmax = h->d.xmin + h->d.dh * (h->X - 1), ymax = h->d.ymin + h->d.dh * (h->Y - 1),
                 zmax = h->d.zmin + h->d.dh * (h->Z - 1);
    for (int i = 0; i < n; i++) {
        const double *c = xyz + 3 * i;
        if (c[0] < h->d.xmin || c[0] > xmax || c[1] < h->d.ymin || c[1] > ymax || c[2] < h->d.zmin || c[2] > zmax)
            return fail(FSI_E_RANGE, "fluid probe %d is not in selected block", i + 1);  // FlowCondition.f90:205-210
    }
    if (int rc = macro_device(h, vf)) return rc;
    if (int rc = out_scratch(h, sizeof(double) * 6 * n)) return rc;
    double *d_xyz = (double *)h->d_out, *d_uvw = d_xyz + 3 * n;
    CK(cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->st));
    CK(launch_probes(h->u, h->X, h->Y, h->Z, h->d.dh, h->d.xmin, h->d.ymin, h->d.zmin, n, d_xyz, Uref, d_uvw, h->st));
    CK(cudaMemcpyAsync(uvw, d_uvw, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->st));
    return check_kerr(h);
}

int fsi_block_initialise(fsi_block_t h, double time) {
    if (!h) return fail(FSI_E_ARG, "null handle");
    Vel v = make_vel(h, time);
    double *dst = (h->esz == 8) ? (double *)h->fa : h->stage;
    CK(launch_init_f64(dst, h->den, h->u, h->X, h->Y, h->Z, h->d.dh, h->d.xmin, h->d.ymin, h->d.zmin, h->d.denIn, v,
                       time, h->st));
    if (h->esz != 8) CK(launch_convert_to_store(h->stage, h->fa, h->N, h->prec, h->st));
    // calculate_SRT_params (FluidDomain.f90:450-456) resets tau_all
    if (h->tau_all) CK(launch_fill_f64(h->tau_all, h->N, h->tau, h->st));
    if (h->tauf) CK(launch_fill_f32(h->tauf, h->N, (float)h->tau, h->st));
    if (h->tauf2) CK(launch_fill_f32(h->tauf2, h->N, (float)h->tau, h->st));
    CK(cudaStreamSynchronize(h->st));
    return FSI_OK;
}

int fsi_block_set_boundary_conditions(fsi_block_t h, double blktime) {
    FSI_CALL_RANGE();
    if (!h) return fail(FSI_E_ARG, "null handle");
    int rc = apply_bcs(h, h->fa, blktime);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->st));
    return FSI_OK;
}

int fsi_block_macro(fsi_block_t h, const double vf[3], double *den, double *uuu) {
    FSI_CALL_RANGE();
    if (!h) return fail(FSI_E_ARG, "null handle");
    double z3[3] = {0, 0, 0};
    const double *v = vf ? vf : z3;
    if (h->esz == 8 && h->prec == FSI_PREC_F64) {
        CK(launch_macro_f64((const double *)h->fa, h->den, h->u, h->X, h->Y, h->Z, h->d.dh, v, h->st));
    } else {
        CK(launch_macro_fast(h->fa, h->prec, h->den, h->u, h->X, h->Y, h->Z, h->d.dh, v, h->st));
    }
    if (den) CK(cudaMemcpyAsync(den, h->den, sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->st));
    if (uuu) CK(cudaMemcpyAsync(uuu, h->u, sizeof(double) * 3 * h->N, cudaMemcpyDeviceToHost, h->st));
    return check_kerr(h);
}

int fsi_block_step(fsi_block_t h, const double vf[3], double blktime) {
    FSI_CALL_RANGE();
    if (!h || !vf) return fail(FSI_E_ARG, "null argument");
    int rc = enqueue_step(h, vf, blktime, true);
    h->win_valid = false;
    return rc;
}

int fsi_block_set_kernel(fsi_block_t h, int kernel) {
    if (!h) return fail(FSI_E_ARG, "null handle");
    if (kernel < FSI_KERNEL_AUTO || kernel > FSI_KERNEL_PIPELINED) return fail(FSI_E_ARG, "unknown kernel %d", kernel);
    if (kernel == FSI_KERNEL_PIPELINED && h->Z % 8 != 0)
        return fail(FSI_E_ARG, "the pipelined kernel needs zDim a multiple of 8");
    if (kernel != h->kernel && h->gexec) {
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    h->kernel = kernel;
    return FSI_OK;
}

int fsi_block_set_ib_mode(fsi_block_t h, int mode) {
    if (!h) return fail(FSI_E_ARG, "null handle");
    if (mode < FSI_IB_AUTO || mode > FSI_IB_GATHER) return fail(FSI_E_ARG, "unknown IB mode %d", mode);
    h->ib_mode = mode;
    return FSI_OK;
}

int fsi_block_timer(fsi_block_t h, int stop, float *ms) {
    if (!h) return fail(FSI_E_ARG, "null handle");
    if (!stop) {
        CK(cudaEventRecord(h->ev0, h->st));
        return FSI_OK;
    }
    CK(cudaEventRecord(h->ev1, h->st));
    CK(cudaEventSynchronize(h->ev1));
    float t = 0.0f;
    CK(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    if (ms) *ms = t;
    return check_kerr(h);
}

int fsi_block_run(fsi_block_t h, const double vf[3], double blktime0, int nsteps, float *ms) {
    FSI_CALL_RANGE();
    if (!h || !vf || nsteps < 0) return fail(FSI_E_ARG, "invalid argument");
    h->win_valid = false;
    // a captured pair of steps is valid when no kernel argument changes from
    // step to step: no boundary depends on time (oscillatory inflow)
    bool time_dep = false;
    for (int k = 0; k < 6; k++) {
        int c = h->d.bndConds[k];
        if (h->d.velocityKind == 2 && (c == BC_EQ || c == BC_NEQ || c == BC_MWALL || c == BC_MWALL_HW)) time_dep = true;
        // the first application of a half-way face only marks it ready
        if ((c == BC_WALL_HW || c == BC_MWALL_HW) && !h->hw_ready[k]) time_dep = true;
    }
    bool use_graph = !time_dep && nsteps >= 2;
    if (use_graph && h->gexec && (memcmp(h->g_vf, vf, sizeof(h->g_vf)) != 0 || h->g_src != h->fa)) {
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    if (use_graph && !h->gexec) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(h, vf, blktime0, false);
        if (!rc) rc = enqueue_step(h, vf, blktime0, false);
        cudaError_t ce = cudaStreamEndCapture(h->st, &g);
        if (rc) return rc;
        if (ce != cudaSuccess) return fail(FSI_E_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        CK(cudaGraphInstantiate(&h->gexec, g, 0));
        cudaGraphDestroy(g);
        memcpy(h->g_vf, vf, sizeof(h->g_vf));
        // capture swapped the buffers twice: the state is unchanged and the
        // graph's first step reads fa
        h->g_src = h->fa;
    }
    CK(cudaEventRecord(h->ev0, h->st));
    int done = 0;
    if (use_graph) {
        // the graph was captured with fa as the source of its first step
        for (; done + 2 <= nsteps; done += 2) CK(cudaGraphLaunch(h->gexec, h->st));
    }
    // an odd remainder (or a time-dependent boundary) runs eagerly
    for (; done < nsteps; done++) {
        int rc = enqueue_step(h, vf, blktime0 + h->d.dh * (double)done, false);
        if (rc) return rc;
    }
    CK(cudaEventRecord(h->ev1, h->st));
    CK(cudaEventSynchronize(h->ev1));
    if (ms) CK(cudaEventElapsedTime(ms, h->ev0, h->ev1));
    return check_kerr(h);
}

// ------------------------------------------------------------------------ IB

int fsi_ib_set_bodies(fsi_block_t h, int nbodies, const int *M, const int bc[6]) {
    if (!h || nbodies < 0 || (nbodies > 0 && !M)) return fail(FSI_E_ARG, "invalid argument");
    if (nbodies > 64) return fail(FSI_E_ARG, "at most 64 bodies per block");
    if (h->ib_pending) return fail(FSI_E_STATE, "an IB step is pending: fsi_block_ib_wait first");
    // every argument checked before the block changes
    long long total = 0;
    for (int b = 0; b < nbodies; b++) {
        if (M[b] <= 0) return fail(FSI_E_ARG, "body %d has no markers", b);
        total += M[b];
        if (total * 64 > 0x7fffffffLL) return fail(FSI_E_ARG, "too many markers");
    }
    // until the new arrays are in place the block has no bodies
    h->nb = 0;
    h->Mtot = 0;
    h->win_valid = false;
    h->M.assign(M, M + nbodies);
    h->offs.assign(nbodies + 1, 0);
    for (int b = 0; b < nbodies; b++) h->offs[b + 1] = h->offs[b] + M[b];
    for (int k = 0; k < 6; k++) h->ibbc[k] = bc ? bc[k] : h->d.bndConds[k];
    void *ptrs[] = {h->d_offs, h->d_xyz, h->d_eforce, h->d_fet, h->d_tolm, h->d_tol, h->d_ei, h->d_ew,
                    h->d_aux, h->d_feat, h->d_c64, h->d_w64};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->h_mk) cudaFreeHost(h->h_mk);
    h->h_mk = nullptr;
    h->d_xyz = h->d_vel = h->d_area = nullptr;
    h->d_aux = nullptr;
    h->d_feat = nullptr;
    h->warm_cap = 0;
    const int Mt = std::max(1, (int)total);
    CK(cudaMalloc((void **)&h->d_offs, sizeof(int) * (nbodies + 1)));
    CK(cudaMalloc((void **)&h->d_xyz, sizeof(double) * 7 * Mt));
    h->d_vel = h->d_xyz + 3 * Mt;
    h->d_area = h->d_xyz + 6 * Mt;
    CK(cudaHostAlloc((void **)&h->h_mk, sizeof(double) * 7 * Mt, cudaHostAllocDefault));
    CK(cudaMalloc((void **)&h->d_eforce, sizeof(double) * 3 * Mt));
    CK(cudaMalloc((void **)&h->d_fet, sizeof(double) * 3 * Mt));
    CK(cudaMalloc((void **)&h->d_tolm, sizeof(double) * Mt));
    CK(cudaMalloc((void **)&h->d_tol, sizeof(double) * 64));
    CK(cudaMalloc((void **)&h->d_ei, sizeof(int16_t) * 12 * Mt));
    CK(cudaMalloc((void **)&h->d_ew, sizeof(float) * 12 * Mt));
    CK(cudaMalloc((void **)&h->d_c64, sizeof(int) * 64 * Mt));
    CK(cudaMalloc((void **)&h->d_w64, sizeof(double) * 64 * Mt));
    CK(cudaMemcpyAsync(h->d_offs, h->offs.data(), sizeof(int) * (nbodies + 1), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->nb = nbodies;
    h->Mtot = (int)total;
    return FSI_OK;
}

namespace {

// The IB window: a box holding every cell any marker's 4x4x4 support can
// reach. Computed on the host from floor((x - xmin)/dh) with a one-cell
// margin on each side (the reference's stencil origin arithmetic,
// Solidbody.f90:771-780, may differ from this estimate by one cell). A box
// that crosses a periodic face spans the whole axis. The stencil kernel
// checks every index against the box.
int compute_window(fsi_block *h, const double *xyz) {
    int lo[3] = {1 << 30, 1 << 30, 1 << 30}, hi[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    const double mins[3] = {h->d.xmin, h->d.ymin, h->d.zmin};
    const int dims[3] = {h->X, h->Y, h->Z};
    for (int m = 0; m < h->Mtot; m++)
        for (int a = 0; a < 3; a++) {
            double v = xyz[3 * m + a];
            if (!std::isfinite(v)) return fail(FSI_E_NAN, "non-finite marker coordinate");
            double t = std::floor((v - mins[a]) / h->d.dh);
            if (t < -1e9 || t > 1e9) return fail(FSI_E_RANGE, "marker far outside the block");
            int i = (int)t;
            lo[a] = std::min(lo[a], i - 2);
            hi[a] = std::max(hi[a], i + 3);
        }
    int box[6];
    for (int a = 0; a < 3; a++) {
        if (lo[a] < 0 || hi[a] > dims[a] - 1) {
            if (h->ibbc[2 * a] == BC_PERIODIC) { lo[a] = 0; hi[a] = dims[a] - 1; }
            else { lo[a] = std::max(lo[a], 0); hi[a] = std::min(hi[a], dims[a] - 1); }
        }
        if (lo[a] > hi[a]) return fail(FSI_E_RANGE, "markers outside the block");
        box[2 * a] = lo[a];
        box[2 * a + 1] = hi[a];
    }
    IbGeom &g = h->geom;
    g.X = h->X; g.Y = h->Y; g.Z = h->Z;
    g.dh = h->d.dh; g.xmin = h->d.xmin; g.ymin = h->d.ymin; g.zmin = h->d.zmin;
    g.invdh = 1.0 / h->d.dh;
    for (int k = 0; k < 6; k++) g.bc[k] = h->ibbc[k];
    g.wx0 = box[0]; g.wx1 = box[1]; g.wy0 = box[2]; g.wy1 = box[3]; g.wz0 = box[4]; g.wz1 = box[5];
    g.WY = box[3] - box[2] + 1;
    g.WZ = box[5] - box[4] + 1;
    h->Nw = (long long)(box[1] - box[0] + 1) * g.WY * g.WZ;
    if (h->Nw > h->Nw_cap) {
        void *ptrs[] = {h->wden, h->wu, h->wforce, h->wu2, h->dlt, h->cnt, h->start, h->fillc};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        long long cap = h->Nw + h->Nw / 2 + 1024;
        CK(cudaMalloc((void **)&h->wden, sizeof(double) * cap));
        CK(cudaMalloc((void **)&h->wu, sizeof(double) * 3 * cap));
        CK(cudaMalloc((void **)&h->wforce, sizeof(double) * 3 * cap));
        CK(cudaMalloc((void **)&h->wu2, sizeof(double) * 3 * cap));
        CK(cudaMalloc((void **)&h->dlt, sizeof(double) * 9 * cap));
        CK(cudaMalloc((void **)&h->cnt, sizeof(int) * cap));
        CK(cudaMalloc((void **)&h->start, sizeof(int) * (cap + 1)));
        CK(cudaMalloc((void **)&h->fillc, sizeof(int) * cap));
        h->Nw_cap = cap;
    }
    long long E = (long long)h->Mtot * 64;
    if (E > h->list_cap) {
        if (h->list) cudaFree(h->list);
        CK(cudaMalloc((void **)&h->list, sizeof(int) * std::max(1LL, E)));
        h->list_cap = E;
    }
    return FSI_OK;
}

// The fast forms: one cooperative launch does the window macro, the stencil,
// the whole penalty loop with its residual test and the spreading; the host
// reads back the Lagrangian force, the iteration count and the residual.
struct Warm {
    const fsi_mlp *mlp = nullptr;  // network of the warm start, or null
    bool aux = false;              // d_aux holds this call's auxiliary inputs
    float *features = nullptr;     // host (12,Mtot) out, or null
    bool seed = false;             // d_eforce holds the caller's initial force
    bool async = false;            // return once queued (fsi_block_ib_wait finishes)
    // queue the fluid step right behind the IB stage (fsi_block_ib_step)
    bool step = false;
    const double *step_vf = nullptr;
    double step_time = 0.0;
    // the IB stage beside the bulk step, already forked onto the second
    // stream (markers uploaded there): its mode
    int forked = 0;
};

// the IB mode fsi_block_ib_step runs for h (FSI_IB_AUTO resolved): OVERLAP
// for the offset forms on the paired kernels (not the gradient models, whose
// velocity pass needs the IB stage's window first), else GRID
int resolve_ib_mode(fsi_block *h, const double vf[3], double blktime) {
    int mode = h->ib_mode;
    if (h->prec == FSI_PREC_F64 || h->prec == FSI_PREC_F64_FAST) return FSI_IB_GRID;
    if (mode == FSI_IB_AUTO) {
        StepArgs t;
        fill_step(h, vf, blktime, true, t);
        mode = (step_fast_paired(t, &h->mm, h->prec, h->d.iCollidModel) && !grad_model(h->d.iCollidModel))
                   ? FSI_IB_OVERLAP : FSI_IB_GRID;
    }
    return mode;
}

// the IB stage's arguments for block h after compute_window (its own marker,
// force, status and residual arrays)
void fill_ib(fsi_block *h, const double vf[3], double denIn, double dt, double Uref, int ntol, double dtol, IbCoop &a) {
    const double ih = 1.0 / h->d.dh;
    a = IbCoop{};
    a.g = h->geom;
    a.N = h->N;
    a.Nw = h->Nw;
    a.f = h->fa;
    for (int k = 0; k < 3; k++) a.vf[k] = vf[k];
    a.nb = h->nb;
    a.Mtot = h->Mtot;
    a.offs = h->d_offs;
    a.xyz = h->d_xyz; a.vel = h->d_vel; a.area = h->d_area;
    a.ei = h->d_ei; a.ew = h->d_ew;
    a.c64 = h->d_c64; a.w64 = h->d_w64;
    a.eforce = h->d_eforce; a.fet = h->d_fet;
    a.wden = h->wden; a.wu = h->wu; a.wforce = h->wforce;
    a.wu2 = h->wu2; a.dlt = h->dlt;
    a.ntol = ntol;
    a.dtol = dtol;
    a.dsumU = (double)h->Mtot * Uref;
    a.invh3p = ((0.5 * dt) * ((ih * ih) * ih)) / denIn;  // Solidbody.f90:996
    a.invh3s = (ih * ih) * ih;                          // Solidbody.f90:936
    a.tol_acc = h->d_tolacc;
    a.status = h->d_status;
    a.res = h->d_res;
    a.Uref = Uref;
}

int ib_check_status(fsi_block *h, int *iters, double *residual, bool keep_window);

// the end of a queued IB step: wait for its force and status copies
int ib_step_finish(fsi_block *h, double *eforce, int *iters, double *residual) {
    CK(cudaEventSynchronize(h->ev_ib));
    if (eforce) memcpy(eforce, h->h_ef, sizeof(double) * 3 * h->Mtot);
    return ib_check_status(h, iters, residual, false);
}

int ib_solve_coop(fsi_block *h, const double vf[3], double denIn, double dt, double Uref, int ntol, double dtol,
                  const Warm &wm, double *eforce, int *iters, double *residual) {
    if (!h->coop_grid) {
        h->coop_grid = ib_coop_grid(h->prec);
        if (h->coop_grid <= 0) return fail(FSI_E_CUDA, "no co-resident grid for the IB kernel");
    }
    if (ntol > h->tolacc_cap) {
        if (h->d_tolacc) cudaFree(h->d_tolacc);
        h->tolacc_cap = std::max(ntol, 64);
        CK(cudaMalloc((void **)&h->d_tolacc, sizeof(double) * h->tolacc_cap));
    }
    // after a stage that did not end cleanly the status words are cleared (a
    // forked stage on the second stream, ahead of it)
    const unsigned bar_base = h->ib_clean ? (unsigned)h->h_stat[2] : 0u;
    if (!h->ib_clean) CK(cudaMemsetAsync(h->d_status, 0, sizeof(int) * 4, wm.forked ? h->st2 : h->st));
    h->ib_clean = false;
    IbCoop a;
    fill_ib(h, vf, denIn, dt, Uref, ntol, dtol, a);
    a.bar_base = bar_base;
    a.mlp = wm.mlp ? wm.mlp->P : nullptr;
    a.mlp_nrm = wm.mlp ? wm.mlp->nrm : nullptr;
    a.aux = wm.aux ? h->d_aux : nullptr;
    a.feat = wm.features ? h->d_feat : nullptr;
    a.Uref = Uref;
    a.seed = wm.seed ? 1 : 0;
    // the IB stage beside the bulk step (fsi_block_ib_step forked it onto the
    // second stream); the window fix-up and the face hooks wait for it
    const int mode = wm.forked;
    if (mode) {
        // the IB stage on one cluster on the second stream, beside the bulk
        // step (both only read the state); the window fix-up and the face
        // hooks wait for it
        if (h->h_ef_cap < h->Mtot) {
            if (h->h_ef) cudaFreeHost(h->h_ef);
            h->h_ef = nullptr;
            h->h_ef_cap = 0;
            CK(cudaHostAlloc((void **)&h->h_ef, sizeof(double) * 3 * h->Mtot, cudaHostAllocDefault));
            h->h_ef_cap = h->Mtot;
        }
        if (mode == FSI_IB_OVERLAP) {
            // beside the bulk step the IB stage takes SM room from it: cap its grid
            long long need = std::max<long long>((h->Mtot + 7) / 8, (h->Nw + 255) / 256);
            long long cap = std::min<long long>(h->coop_grid, std::max<long long>(FSI_IB_OVERLAP_CTAS, need / 6));
            CK(launch_ib_coop(a, h->prec, (int)std::max<long long>(1, std::min<long long>(need, cap)), h->st2));
        } else {
            CK(launch_ib_cluster(a, h->prec, h->st2));
        }
        // the window fix-up waits for the kernel only, not for the copies
        CK(cudaEventRecord(h->ev_ibk, h->st2));
        CK(cudaMemcpyAsync(h->h_ef, h->d_eforce, sizeof(double) * 3 * h->Mtot, cudaMemcpyDeviceToHost, h->st2));
        CK(cudaMemcpyAsync(h->h_stat, h->d_status, STAT_BYTES, cudaMemcpyDeviceToHost, h->st2));
        CK(cudaEventRecord(h->ev_ib, h->st2));
        h->win_valid = true;
        int rc = enqueue_step(h, wm.step_vf, wm.step_time, true, h->ev_ibk);
        h->win_valid = false;
        if (rc) return rc;
    } else {
    // one warp per marker in the penalty loop and a thread per window cell in
    // the macro phase are all the parallelism there is; a smaller grid makes
    // each of the grid barriers cheaper
    long long need = std::max<long long>((h->Mtot + 7) / 8, (h->Nw + 255) / 256);
    const int grid = (int)std::max<long long>(1, std::min<long long>(need, h->coop_grid));
    CK(launch_ib_coop(a, h->prec, grid, h->st));
    if (wm.step) {
        // force, status and residual into pinned staging on the second
        // stream, while the fluid step follows the IB stage on this one; the
        // host waits for the copies only
        if (h->h_ef_cap < h->Mtot) {
            if (h->h_ef) cudaFreeHost(h->h_ef);
            h->h_ef = nullptr;
            h->h_ef_cap = 0;
            CK(cudaHostAlloc((void **)&h->h_ef, sizeof(double) * 3 * h->Mtot, cudaHostAllocDefault));
            h->h_ef_cap = h->Mtot;
        }
        CK(cudaEventRecord(h->ev_ibk, h->st));
        CK(cudaStreamWaitEvent(h->st2, h->ev_ibk, 0));
        CK(cudaMemcpyAsync(h->h_ef, h->d_eforce, sizeof(double) * 3 * h->Mtot, cudaMemcpyDeviceToHost, h->st2));
        CK(cudaMemcpyAsync(h->h_stat, h->d_status, STAT_BYTES, cudaMemcpyDeviceToHost, h->st2));
        CK(cudaEventRecord(h->ev_ib, h->st2));
        h->win_valid = true;
        int rc = enqueue_step(h, wm.step_vf, wm.step_time, true);
        h->win_valid = false;
        if (rc) return rc;
    } else {
        CK(cudaMemcpyAsync(eforce, h->d_eforce, sizeof(double) * 3 * h->Mtot, cudaMemcpyDeviceToHost, h->st));
        if (wm.features)
            CK(cudaMemcpyAsync(wm.features, h->d_feat, sizeof(float) * 12 * h->Mtot, cudaMemcpyDeviceToHost, h->st));
        CK(cudaMemcpyAsync(h->h_stat, h->d_status, STAT_BYTES, cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
    }
    }
    if (wm.step) {
        if (wm.async) {
            h->ib_pending = 1;
            return FSI_OK;
        }
        return ib_step_finish(h, eforce, iters, residual);
    }
    return ib_check_status(h, iters, residual, true);
}

// the status of the last IB stage (its copy in h_stat): error codes, the
// iteration count and the residual
int ib_check_status(fsi_block *h, int *iters, double *residual, bool keep_window) {
    if (h->h_stat[4]) return fail(FSI_E_TIMEOUT, "step kernel: a bounded wait ran out");
    const int st = h->h_stat[0];
    if (st & 1) return fail(FSI_E_RANGE, "index out of block bounds in IB stencil");
    if (st & 2) return fail(FSI_E_RANGE, "IB stencil outside the IB window");
    if (st & 4) return fail(FSI_E_NAN, "Nan found in PenaltyForce");
    if (st & 8) return fail(FSI_E_TIMEOUT, "IB grid barrier timed out");
    const int it = h->h_stat[1];
    if (iters) *iters = it;
    if (residual) *residual = *(const double *)(h->h_stat + 8);
    h->win_valid = keep_window;
    h->ib_clean = st == 0;
    return FSI_OK;
}

// the window and the marker arrays of one solve
int ib_upload(fsi_block *h, const double *xyz, const double *vel, const double *area, cudaStream_t st = nullptr) {
    int rc = compute_window(h, xyz);
    if (rc) return rc;
    const int Mt = h->Mtot;
    if (!st) st = h->st;
    // through the pinned mirror: every caller waits for its IB stage (which
    // follows this copy on the stream) before it returns, so the mirror is
    // free again when the next call fills it
    memcpy(h->h_mk, xyz, sizeof(double) * 3 * Mt);
    memcpy(h->h_mk + 3 * Mt, vel, sizeof(double) * 3 * Mt);
    memcpy(h->h_mk + 6 * Mt, area, sizeof(double) * Mt);
    CK(cudaMemcpyAsync(h->d_xyz, h->h_mk, sizeof(double) * 7 * Mt, cudaMemcpyHostToDevice, st));
    return FSI_OK;
}

}  // namespace

int fsi_ib_solve(fsi_block_t h, const double *xyz, const double *vel, const double *area, const double vf[3],
                 double denIn, double dt, double Uref, int ntol, double dtol, double *eforce, int *iters,
                 double *residual) {
    FSI_CALL_RANGE();
    if (!h || !vf) return fail(FSI_E_ARG, "null argument");
    if (h->ib_pending) return fail(FSI_E_STATE, "an IB step is pending: fsi_block_ib_wait first");
    h->win_valid = false;
    if (iters) *iters = 0;
    if (residual) *residual = 0.0;
    if (h->nb == 0 || h->Mtot == 0) return FSI_OK;
    if (!xyz || !vel || !area || !eforce) return fail(FSI_E_ARG, "null marker array");
    int rc = ib_upload(h, xyz, vel, area);
    if (rc) return rc;
    const int Mt = h->Mtot;
    // the fast forms' cooperative stage, unless the gather kernels are asked for
    if (h->prec != FSI_PREC_F64 && h->ib_mode != FSI_IB_GATHER)
        return ib_solve_coop(h, vf, denIn, dt, Uref, ntol, dtol, Warm{}, eforce, iters, residual);
    CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->st));
    CK(cudaMemsetAsync(h->d_eforce, 0, sizeof(double) * 3 * Mt, h->st));
    // calculate_macro_quantities_ + ResetVolumeForce_ restricted to the window
    if (h->prec == FSI_PREC_F64) CK(launch_win_macro_f64(h->fa, h->prec, h->wden, h->wu, h->geom, h->N, vf, h->st));
    else CK(launch_win_macro_fast(h->fa, h->prec, h->wden, h->wu, h->geom, h->N, vf, h->st));
    CK(launch_ib_stencil(h->d_xyz, h->d_offs, h->nb, Mt, h->geom, h->d_ei, h->d_ew, h->d_err, h->st));
    CK(launch_ib_csr(h->d_ei, Mt, h->geom, h->Nw, h->cnt, h->start, h->fillc, h->list, h->st));
    // PenaltyForce_ constants, Solidbody.f90:996 and :936
    const double ih = 1.0 / h->d.dh;
    const double invh3p = ((0.5 * dt) * ((ih * ih) * ih)) / denIn;
    const double invh3s = (ih * ih) * ih;
    int it = 0;
    double dmax = 1e10;
    CK(cudaMemcpyAsync(h->h_err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (*h->h_err) {
        return fail(FSI_E_RANGE, (*h->h_err & 1) ? "index out of block bounds in IB stencil"
                                                 : "IB stencil outside the IB window");
    }
    while (it < ntol && dmax > dtol) {
        for (int b = 0; b < h->nb; b++) {
            int m0 = h->offs[b], m1 = h->offs[b + 1];
            CK(launch_ib_interp(h->d_ei, h->d_ew, h->d_vel, h->d_area, h->wu, h->geom, m0, m1, invh3p, h->d_eforce,
                                h->d_fet, h->d_tolm, h->st));
            CK(launch_ib_reduce(h->d_tolm, m0, m1, h->d_tol + b, h->st));
            CK(launch_ib_correct(h->d_ew, h->start, h->list, h->Nw, m0, m1, h->d_fet, h->wu, h->st));
        }
        CK(cudaMemcpyAsync(h->h_tol, h->d_tol, sizeof(double) * h->nb, cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        // calculate_interaction_force, Solidbody.f90:896-905
        dmax = 0.0;
        double dsum = 0.0;
        for (int b = 0; b < h->nb; b++) {
            if (!std::isfinite(h->h_tol[b])) return fail(FSI_E_NAN, "Nan found in PenaltyForce");
            dmax = dmax + h->h_tol[b];
            dsum = dsum + (double)h->M[b];
        }
        dmax = dmax / (dsum * Uref);
        it = it + 1;
    }
    CK(launch_ib_spread(h->d_ew, h->start, h->list, h->Nw, h->d_eforce, invh3s, vf, h->wforce, h->st));
    CK(cudaMemcpyAsync(eforce, h->d_eforce, sizeof(double) * 3 * Mt, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (iters) *iters = it;
    if (residual) *residual = dmax;
    h->win_valid = true;
    return FSI_OK;
}

int fsi_ib_solve_warm(fsi_block_t h, const double *xyz, const double *vel, const double *area, const double *aux,
                      const double vf[3], double denIn, double dt, double Uref, int ntol, double dtol, fsi_mlp_t warm,
                      float *features, double *eforce, int *iters, double *residual) {
    FSI_CALL_RANGE();
    if (!h || !vf) return fail(FSI_E_ARG, "null argument");
    if (h->ib_pending) return fail(FSI_E_STATE, "an IB step is pending: fsi_block_ib_wait first");
    if (h->prec == FSI_PREC_F64)
        return fail(FSI_E_ARG, "the warm start needs a fast form; FSI_PREC_F64 keeps the reference's iteration");
    if (warm && !warm->norm_set) return fail(FSI_E_STATE, "network statistics not set (fsi_mlp_set_norm)");
    if (!(Uref > 0.0)) return fail(FSI_E_ARG, "Uref must be positive");
    if (warm) {
        int dev = -1;
        CK(cudaGetDevice(&dev));
        if (dev != warm->dev) return fail(FSI_E_ARG, "network lives on device %d, block on %d", warm->dev, dev);
    }
    h->win_valid = false;
    if (iters) *iters = 0;
    if (residual) *residual = 0.0;
    if (h->nb == 0 || h->Mtot == 0) return FSI_OK;
    if (!xyz || !vel || !area || !eforce) return fail(FSI_E_ARG, "null marker array");
    int rc = ib_upload(h, xyz, vel, area);
    if (rc) return rc;
    if (h->warm_cap < h->Mtot) {
        if (h->d_aux) cudaFree(h->d_aux);
        if (h->d_feat) cudaFree(h->d_feat);
        h->d_aux = nullptr;
        h->d_feat = nullptr;
        h->warm_cap = 0;
        CK(cudaMalloc((void **)&h->d_aux, sizeof(double) * 6 * h->Mtot));
        CK(cudaMalloc((void **)&h->d_feat, sizeof(float) * 12 * h->Mtot));
        h->warm_cap = h->Mtot;
    }
    if (aux) CK(cudaMemcpyAsync(h->d_aux, aux, sizeof(double) * 6 * h->Mtot, cudaMemcpyHostToDevice, h->st));
    Warm wm;
    wm.mlp = warm;
    wm.aux = aux != nullptr;
    wm.features = features;
    return ib_solve_coop(h, vf, denIn, dt, Uref, ntol, dtol, wm, eforce, iters, residual);
}

int fsi_ib_solve_seeded(fsi_block_t h, const double *xyz, const double *vel, const double *area, const double *guess,
                        const double vf[3], double denIn, double dt, double Uref, int ntol, double dtol, double *eforce,
                        int *iters, double *residual) {
    FSI_CALL_RANGE();
    if (!h || !vf) return fail(FSI_E_ARG, "null argument");
    if (h->ib_pending) return fail(FSI_E_STATE, "an IB step is pending: fsi_block_ib_wait first");
    if (h->prec == FSI_PREC_F64)
        return fail(FSI_E_ARG, "the seeded start needs a fast form; FSI_PREC_F64 keeps the reference's iteration");
    h->win_valid = false;
    if (iters) *iters = 0;
    if (residual) *residual = 0.0;
    if (h->nb == 0 || h->Mtot == 0) return FSI_OK;
    if (!xyz || !vel || !area || !guess || !eforce) return fail(FSI_E_ARG, "null marker array");
    for (long long k = 0; k < 3LL * h->Mtot; k++)
        if (!std::isfinite(guess[k])) return fail(FSI_E_NAN, "non-finite initial force");
    int rc = ib_upload(h, xyz, vel, area);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->d_eforce, guess, sizeof(double) * 3 * h->Mtot, cudaMemcpyHostToDevice, h->st));
    Warm wm;
    wm.seed = true;
    return ib_solve_coop(h, vf, denIn, dt, Uref, ntol, dtol, wm, eforce, iters, residual);
}

}  // extern "C"

namespace {

// fsi_block_ib_step and its queued form
int ib_step_impl(fsi_block_t h, const double *xyz, const double *vel, const double *area, const double vf[3],
                 double denIn, double dt, double Uref, int ntol, double dtol, double blktime, double *eforce,
                 int *iters, double *residual, bool async) {
    if (!h || !vf) return fail(FSI_E_ARG, "null argument");
    if (h->ib_pending) return fail(FSI_E_STATE, "an IB step is pending: fsi_block_ib_wait first");
    if (h->prec == FSI_PREC_F64 || h->ib_mode == FSI_IB_GATHER || h->nb == 0 || h->Mtot == 0) {
        if (!async) {
            int rc = fsi_ib_solve(h, xyz, vel, area, vf, denIn, dt, Uref, ntol, dtol, eforce, iters, residual);
            if (rc) return rc;
            return fsi_block_step(h, vf, blktime);
        }
        // the exact form runs the two calls one after the other; the force
        // waits in the staging buffer for fsi_block_ib_wait
        if (h->h_ef_cap < h->Mtot) {
            if (h->h_ef) cudaFreeHost(h->h_ef);
            h->h_ef = nullptr;
            h->h_ef_cap = 0;
            CK(cudaHostAlloc((void **)&h->h_ef, sizeof(double) * 3 * h->Mtot, cudaHostAllocDefault));
            h->h_ef_cap = h->Mtot;
        }
        int it = 0;
        double res = 0.0;
        int rc = fsi_ib_solve(h, xyz, vel, area, vf, denIn, dt, Uref, ntol, dtol, h->h_ef, &it, &res);
        if (rc) return rc;
        rc = fsi_block_step(h, vf, blktime);
        if (rc) return rc;
        h->pend_iters = it;
        h->pend_res = res;
        h->ib_pending = 2;
        return FSI_OK;
    }
    h->win_valid = false;
    if (iters) *iters = 0;
    if (residual) *residual = 0.0;
    if (!xyz || !vel || !area || (!eforce && !async)) return fail(FSI_E_ARG, "null marker array");
    Warm wm;
    wm.step = true;
    wm.async = async;
    wm.step_vf = vf;
    wm.step_time = blktime;
    const int mode = resolve_ib_mode(h, vf, blktime);
    cudaStream_t ust = h->st;
    if (mode == FSI_IB_OVERLAP || mode == FSI_IB_CLUSTER) {
        // the IB stage beside the bulk step: fork after the previous step, and
        // keep the marker uploads off the bulk step's stream as well
        CK(cudaEventRecord(h->ev_fork, h->st));
        CK(cudaStreamWaitEvent(h->st2, h->ev_fork, 0));
        ust = h->st2;
        wm.forked = mode;
    }
    int rc = ib_upload(h, xyz, vel, area, ust);
    if (rc) return rc;
    return ib_solve_coop(h, vf, denIn, dt, Uref, ntol, dtol, wm, eforce, iters, residual);
}

}  // namespace

extern "C" {

int fsi_block_ib_step(fsi_block_t h, const double *xyz, const double *vel, const double *area, const double vf[3],
                      double denIn, double dt, double Uref, int ntol, double dtol, double blktime, double *eforce,
                      int *iters, double *residual) {
    FSI_CALL_RANGE();
    return ib_step_impl(h, xyz, vel, area, vf, denIn, dt, Uref, ntol, dtol, blktime, eforce, iters, residual, false);
}

int fsi_block_ib_step_async(fsi_block_t h, const double *xyz, const double *vel, const double *area,
                            const double vf[3], double denIn, double dt, double Uref, int ntol, double dtol,
                            double blktime) {
    FSI_CALL_RANGE();
    return ib_step_impl(h, xyz, vel, area, vf, denIn, dt, Uref, ntol, dtol, blktime, nullptr, nullptr, nullptr,
                        true);
}

int fsi_block_ib_wait(fsi_block_t h, double *eforce, int *iters, double *residual) {
    FSI_CALL_RANGE();
    if (!h) return fail(FSI_E_ARG, "null handle");
    const int mode = h->ib_pending;
    if (!mode) return fail(FSI_E_STATE, "no IB step pending (fsi_block_ib_step_async)");
    h->ib_pending = 0;
    if (mode == 2) {
        if (eforce && h->Mtot) memcpy(eforce, h->h_ef, sizeof(double) * 3 * h->Mtot);
        if (iters) *iters = h->pend_iters;
        if (residual) *residual = h->pend_res;
        return FSI_OK;
    }
    return ib_step_finish(h, eforce, iters, residual);
}

int fsi_ib_get_stencil(fsi_block_t h, int16_t *ei, float *ew) {
    if (!h) return fail(FSI_E_ARG, "null handle");
    if (h->Mtot == 0) return FSI_OK;
    if (ei) CK(cudaMemcpyAsync(ei, h->d_ei, sizeof(int16_t) * 12 * h->Mtot, cudaMemcpyDeviceToHost, h->st));
    if (ew) CK(cudaMemcpyAsync(ew, h->d_ew, sizeof(float) * 12 * h->Mtot, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return FSI_OK;
}

int fsi_ib_get_window(fsi_block_t h, int box[6]) {
    if (!h || !box) return fail(FSI_E_ARG, "null argument");
    box[0] = h->geom.wx0; box[1] = h->geom.wx1; box[2] = h->geom.wy0;
    box[3] = h->geom.wy1; box[4] = h->geom.wz0; box[5] = h->geom.wz1;
    return FSI_OK;
}

// ---------------------------------------------------------- block refinement

}  // extern "C"

namespace {
int static_scratch(double **out);  // the allocation-free variant's scratch, end of this file
}  // namespace

extern "C" {

int fsi_pair_create(fsi_pair_t *out, fsi_block_t fa, fsi_block_t so, int scheme) {
    if (!out || !fa || !so) return fail(FSI_E_ARG, "null argument");
    *out = nullptr;
    if (fa->prec != so->prec) return fail(FSI_E_ARG, "father and son share one storage form");
    fsi_pair *p = new (std::nothrow) fsi_pair();
    if (!p) return fail(FSI_E_ARG, "out of host memory");
    p->fa = fa;
    p->so = so;
    p->scheme = scheme;
    PairGeom &g = p->p;
    // build_blocks_comunication, LBMBlockComm.f90:48-91
    for (int j = 0; j < 6; j++) g.sds[j] = (so->d.bndConds[j] == BC_FLUID) ? ((j % 2 == 0) ? 1 : -1) : 0;
    int sxD = so->X - so->periodic[0], syD = so->Y - so->periodic[1], szD = so->Z - so->periodic[2];
    g.s[0] = 1; g.s[2] = 1; g.s[4] = 1;
    g.s[1] = sxD; g.s[3] = syD; g.s[5] = szD;
    g.f[0] = (int)floor((so->d.xmin - fa->d.xmin) / fa->d.dh + 1.5);
    g.f[2] = (int)floor((so->d.ymin - fa->d.ymin) / fa->d.dh + 1.5);
    g.f[4] = (int)floor((so->d.zmin - fa->d.zmin) / fa->d.dh + 1.5);
    int ratio = (int)floor(fa->d.dh / so->d.dh + 0.5);
    if (ratio != 2) { delete p; return fail(FSI_E_ARG, "refinement ratio must be 2 (m_gridDelta)"); }
    g.f[1] = g.f[0] + (sxD - 1) / ratio;
    g.f[3] = g.f[2] + (syD - 1) / ratio;
    g.f[5] = g.f[4] + (szD - 1) / ratio;
    for (int j = 0; j < 6; j++) { g.si[j] = g.s[j] + g.sds[j] * ratio; g.fi[j] = g.f[j] + g.sds[j]; }
    g.xDimS = so->X; g.xDimF = g.f[1] - g.f[0] + 1;
    g.yDimS = so->Y; g.yDimF = g.f[3] - g.f[2] + 1;
    g.zDimS = so->Z; g.zDimF = g.f[5] - g.f[4] + 1;
    if (g.f[0] < 1 || g.f[2] < 1 || g.f[4] < 1 || g.f[1] > fa->X || g.f[3] > fa->Y || g.f[5] > fa->Z) {
        delete p;
        return fail(FSI_E_ARG, "son block does not lie inside its father");
    }
    // interpolate_fIn (LBMBlockComm.f90:808-956) reads father face node
    // (n+1)/2 for the last odd son node n of a face direction, and the
    // third/fourth-order stencil reaches three son nodes and two father nodes
    // past its own: on narrower faces (son faces under 5 nodes a side, or a
    // son periodic along an odd face direction) the reference reads outside
    // its face arrays. Such pairs are refused here rather than left to read
    // whatever lies next to the face.
    for (int k = 0; k < 6; k++) {
        if (so->d.bndConds[k] != BC_FLUID) continue;
        int ax = k >> 1;
        int AF = ax == 2 ? g.yDimF : g.zDimF, BF = ax == 0 ? g.yDimF : g.xDimF;
        int AS = ax == 2 ? g.yDimS : g.zDimS, BS = ax == 0 ? g.yDimS : g.xDimS;
        int AO = (AS % 2) ? AS : AS - 1, BO = (BS % 2) ? BS : BS - 1;  // last odd son node
        bool ok = (AO + 1) / 2 <= AF && (BO + 1) / 2 <= BF;
        if (scheme == 2) ok = ok && AS >= 5 && BS >= 5;
        if (!ok) {
            delete p;
            return fail(FSI_E_ARG,
                        "son face %d (%d x %d nodes, father %d x %d) is too narrow for interpolation scheme %d: "
                        "the reference's stencil would read outside the face",
                        k, AS, BS, AF, BF, scheme);
        }
    }
    size_t maxS = 0;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 6; k++) {
        if (so->d.bndConds[k] != BC_FLUID) continue;
        int ax = k >> 1;
        size_t AF = ax == 2 ? g.yDimF : g.zDimF, BF = ax == 0 ? g.yDimF : g.xDimF;
        size_t AS = ax == 2 ? g.yDimS : g.zDimS, BS = ax == 0 ? g.yDimS : g.xDimS;
        maxS = std::max(maxS, AS * BS);
        for (int t = 0; t < 2; t++) {
            if (e == cudaSuccess) e = cudaMalloc((void **)&p->buf[k][t], sizeof(double) * 19 * AF * BF);
            if (e == cudaSuccess) e = cudaMalloc((void **)&p->buft[k][t], sizeof(double) * AF * BF);
        }
    }
    if (maxS) {
        if (e == cudaSuccess) e = cudaMalloc((void **)&p->scr_f, sizeof(double) * 19 * maxS);
        if (e == cudaSuccess) e = cudaMalloc((void **)&p->scr_t, sizeof(double) * maxS);
    }
    p->scr_cells = (long long)maxS;
    if (e == cudaSuccess) e = cudaMalloc((void **)&p->d_err, sizeof(int) * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->d_err, 0, sizeof(int) * 4, fa->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(fa->st);
    if (e != cudaSuccess) {
        fsi_pair_destroy(p);
        return fail(FSI_E_CUDA, "pair allocation: %s", cudaGetErrorString(e));
    }
    // Place the static scratch of fsi_pair_father_to_son_static on this device
    // now, at set-up: under lazy module loading the array's module (and its
    // memory) would otherwise load at the first static call, inside the
    // host's time loop.
    double *scr = nullptr;
    int rc = static_scratch(&scr);
    if (rc) {
        fsi_pair_destroy(p);
        return rc;
    }
    *out = p;
    return FSI_OK;
}

int fsi_pair_destroy(fsi_pair_t p) {
    if (!p) return FSI_OK;
    for (int k = 0; k < 6; k++)
        for (int t = 0; t < 2; t++) {
            if (p->buf[k][t]) cudaFree(p->buf[k][t]);
            if (p->buft[k][t]) cudaFree(p->buft[k][t]);
        }
    if (p->scr_f) cudaFree(p->scr_f);
    if (p->scr_t) cudaFree(p->scr_t);
    if (p->d_err) cudaFree(p->d_err);
    delete p;
    return FSI_OK;
}

}  // extern "C"

namespace {
// reads and clears the pair's error word after its stream has drained
int pair_check(fsi_pair *p) {
    int h[3] = {0, 0, 0};
    cudaStream_t st = p->fa->st;
    CK(cudaMemcpyAsync(h, p->d_err, sizeof(int) * 3, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h[0] == 0) return FSI_OK;
    CK(cudaMemsetAsync(p->d_err, 0, sizeof(int) * 4, st));
    CK(cudaStreamSynchronize(st));
    long long idx = (long long)(unsigned)h[1] | ((long long)h[2] << 32);
    static const char *what[] = {"", "interpolation source", "interpolation target", "son face cell",
                                 "father face cell", "son cell", "father cell"};
    return fail(FSI_E_RANGE, "block refinement: %s index %lld out of range", what[h[0] >= 1 && h[0] <= 6 ? h[0] : 0],
                idx);
}
}  // namespace

extern "C" {

int fsi_pair_extract(fsi_pair_t p, int time_level) {
    FSI_CALL_RANGE();
    if (!p || (time_level != 1 && time_level != 2)) return fail(FSI_E_ARG, "invalid argument");
    fsi_block *fa = p->fa;
    for (int k = 0; k < 6; k++) {
        if (p->so->d.bndConds[k] != BC_FLUID) continue;
        CK(launch_pair_extract(fa->fa, fa->prec, fa->X, fa->Y, fa->Z, tau_src(fa), p->p, k, p->buf[k][time_level - 1],
                               p->buft[k][time_level - 1], p->d_err, fa->st));
        if (time_level == 2) {
            int ax = k >> 1;
            long long A = ax == 2 ? p->p.yDimF : p->p.zDimF, B = ax == 0 ? p->p.yDimF : p->p.xDimF;
            CK(launch_pair_average(p->buf[k][0], p->buf[k][1], 19 * A * B, fa->st));
            CK(launch_pair_average(p->buft[k][0], p->buft[k][1], A * B, fa->st));
        }
    }
    CK(cudaStreamSynchronize(fa->st));
    return pair_check(p);
}

int fsi_pair_father_to_son(fsi_pair_t p, int n_timeStep, const double vf[3]) {
    FSI_CALL_RANGE();
    if (!p || !vf) return fail(FSI_E_ARG, "invalid argument");
    fsi_block *so = p->so, *fa = p->fa;
    CK(cudaStreamSynchronize(fa->st));
    for (int k = 0; k < 6; k++) {
        if (p->p.sds[k] == 0) continue;
        int lvl = (n_timeStep == 0) ? 0 : 1;
        CK(launch_pair_f2s(so->fa, so->prec, so->X, so->Y, so->Z, tau_src(so), p->p, k, p->buf[k][lvl], p->buft[k][lvl],
                           p->scheme, p->scr_f, p->scr_t, p->scr_cells, vf, fa->d.dh, p->d_err, so->st));
    }
    CK(cudaStreamSynchronize(so->st));
    return pair_check(p);
}

int fsi_pair_son_to_father(fsi_pair_t p, const double vf[3]) {
    FSI_CALL_RANGE();
    if (!p || !vf) return fail(FSI_E_ARG, "invalid argument");
    fsi_block *so = p->so, *fa = p->fa;
    CK(cudaStreamSynchronize(so->st));
    for (int k = 0; k < 6; k++) {
        int want = (k % 2 == 0) ? 1 : -1;
        if (p->p.sds[k] != want) continue;
        CK(launch_pair_s2f(fa->fa, fa->prec, fa->X, fa->Y, fa->Z, tau_src(fa), so->fa, so->X, so->Y, so->Z, tau_src(so),
                           p->p, k, vf, so->d.dh, p->d_err, fa->st));
    }
    CK(cudaStreamSynchronize(fa->st));
    return pair_check(p);
}

}  // extern "C"

// ------------------------------------------------------------- warm start

namespace {

uint64_t splitmix64(uint64_t &x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double unit_uniform(uint64_t &x) { return (double)(splitmix64(x) >> 11) * (1.0 / 9007199254740992.0); }

void free_mlp(fsi_mlp *m) {
    if (!m) return;
    void *ptrs[] = {m->P, m->nrm, m->grad, m->m, m->v, m->loss, m->X, m->Y, m->perm};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (m->hperm) cudaFreeHost(m->hperm);
    for (int k = 0; k < 2; k++)
        if (m->ev[k]) cudaEventDestroy(m->ev[k]);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
}

int mlp_reserve(fsi_mlp *m, long long n) {
    if (n <= m->cap) return FSI_OK;
    CK(cudaStreamSynchronize(m->st));
    void *ptrs[] = {m->X, m->Y, m->perm};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (m->hperm) cudaFreeHost(m->hperm);
    m->X = m->Y = nullptr;
    m->perm = m->hperm = nullptr;
    m->cap = 0;
    CK(cudaMalloc((void **)&m->X, sizeof(float) * FSI_MLP_IN * n));
    CK(cudaMalloc((void **)&m->Y, sizeof(float) * FSI_MLP_OUT * n));
    CK(cudaMalloc((void **)&m->perm, sizeof(int) * 2 * n));
    CK(cudaMallocHost((void **)&m->hperm, sizeof(int) * 2 * n));
    m->cap = n;
    return FSI_OK;
}

int mlp_reset_adam(fsi_mlp *m) {
    CK(cudaMemsetAsync(m->grad, 0, sizeof(float) * FSI_MLP_NPARAM, m->st));
    CK(cudaMemsetAsync(m->m, 0, sizeof(float) * FSI_MLP_NPARAM, m->st));
    CK(cudaMemsetAsync(m->v, 0, sizeof(float) * FSI_MLP_NPARAM, m->st));
    m->t = 0;
    return FSI_OK;
}

int mlp_create(fsi_mlp *m, unsigned long long seed) {
    CK(cudaGetDevice(&m->dev));
    CK(cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking));
    for (int k = 0; k < 2; k++) CK(cudaEventCreateWithFlags(&m->ev[k], cudaEventDisableTiming));
    float **bufs[] = {&m->P, &m->grad, &m->m, &m->v};
    for (float **b : bufs) CK(cudaMalloc((void **)b, sizeof(float) * FSI_MLP_NPARAM));
    CK(cudaMalloc((void **)&m->nrm, sizeof(float) * FSI_MLP_NNORM));
    m->loss_cap = 64;
    CK(cudaMalloc((void **)&m->loss, sizeof(float) * m->loss_cap));
    // Glorot-uniform weights, zero biases
    std::vector<float> P(FSI_MLP_NPARAM, 0.0f);
    uint64_t r = seed;
    const int fan[3][2] = {{FSI_MLP_IN, MLP_H}, {MLP_H, MLP_H}, {MLP_H, FSI_MLP_OUT}};
    const int w0[3] = {MLP_W1, MLP_W2, MLP_W3};
    for (int l = 0; l < 3; l++) {
        const double lim = std::sqrt(6.0 / (fan[l][0] + fan[l][1]));
        for (int i = 0; i < fan[l][0] * fan[l][1]; i++) P[w0[l] + i] = (float)((2.0 * unit_uniform(r) - 1.0) * lim);
    }
    CK(cudaMemcpyAsync(m->P, P.data(), sizeof(float) * FSI_MLP_NPARAM, cudaMemcpyHostToDevice, m->st));
    std::vector<float> nrm(FSI_MLP_NNORM, 0.0f);
    for (int k = 0; k < FSI_MLP_IN; k++) nrm[FSI_MLP_IN + k] = 1.0f;
    for (int c = 0; c < FSI_MLP_OUT; c++) nrm[2 * FSI_MLP_IN + FSI_MLP_OUT + c] = 1.0f;
    CK(cudaMemcpyAsync(m->nrm, nrm.data(), sizeof(float) * FSI_MLP_NNORM, cudaMemcpyHostToDevice, m->st));
    if (int rc = mlp_reset_adam(m)) return rc;
    CK(cudaStreamSynchronize(m->st));
    return FSI_OK;
}

}  // namespace

extern "C" {

int fsi_mlp_create(fsi_mlp_t *out, unsigned long long seed) {
    if (!out) return fail(FSI_E_ARG, "null argument");
    *out = nullptr;
    fsi_mlp *m = new (std::nothrow) fsi_mlp;
    if (!m) return fail(FSI_E_ARG, "out of host memory");
    if (int rc = mlp_create(m, seed)) {
        free_mlp(m);
        return rc;
    }
    *out = m;
    return FSI_OK;
}

int fsi_mlp_destroy(fsi_mlp_t m) {
    if (!m) return FSI_OK;
    cudaStreamSynchronize(m->st);
    free_mlp(m);
    return FSI_OK;
}

int fsi_mlp_set_params(fsi_mlp_t m, const float *params, int n) {
    if (!m || !params) return fail(FSI_E_ARG, "null argument");
    if (n != FSI_MLP_NPARAM) return fail(FSI_E_ARG, "expected %d parameters, got %d", FSI_MLP_NPARAM, n);
    CK(cudaMemcpyAsync(m->P, params, sizeof(float) * n, cudaMemcpyHostToDevice, m->st));
    if (int rc = mlp_reset_adam(m)) return rc;
    CK(cudaStreamSynchronize(m->st));
    return FSI_OK;
}

int fsi_mlp_get_params(fsi_mlp_t m, float *params, int n) {
    if (!m || !params) return fail(FSI_E_ARG, "null argument");
    if (n != FSI_MLP_NPARAM) return fail(FSI_E_ARG, "expected %d parameters, got %d", FSI_MLP_NPARAM, n);
    CK(cudaMemcpyAsync(params, m->P, sizeof(float) * n, cudaMemcpyDeviceToHost, m->st));
    CK(cudaStreamSynchronize(m->st));
    return FSI_OK;
}

int fsi_mlp_set_norm(fsi_mlp_t m, const float *norm) {
    if (!m || !norm) return fail(FSI_E_ARG, "null argument");
    for (int k = 0; k < FSI_MLP_NNORM; k++)
        if (!std::isfinite(norm[k])) return fail(FSI_E_ARG, "non-finite statistic %d", k);
    for (int k = 0; k < FSI_MLP_IN; k++)
        if (!(norm[FSI_MLP_IN + k] > 0.0f)) return fail(FSI_E_ARG, "input deviation %d must be positive", k);
    for (int c = 0; c < FSI_MLP_OUT; c++)
        if (!(norm[2 * FSI_MLP_IN + FSI_MLP_OUT + c] > 0.0f))
            return fail(FSI_E_ARG, "output deviation %d must be positive", c);
    CK(cudaMemcpyAsync(m->nrm, norm, sizeof(float) * FSI_MLP_NNORM, cudaMemcpyHostToDevice, m->st));
    CK(cudaStreamSynchronize(m->st));
    m->norm_set = true;
    return FSI_OK;
}

int fsi_mlp_forward(fsi_mlp_t m, const float *x, int n, float *y) {
    if (!m || n < 0 || (n > 0 && (!x || !y))) return fail(FSI_E_ARG, "invalid argument");
    if (!m->norm_set) return fail(FSI_E_STATE, "network statistics not set (fsi_mlp_set_norm)");
    if (n == 0) return FSI_OK;
    if (int rc = mlp_reserve(m, n)) return rc;
    CK(cudaMemcpyAsync(m->X, x, sizeof(float) * FSI_MLP_IN * n, cudaMemcpyHostToDevice, m->st));
    CK(launch_mlp_forward(m->P, m->nrm, m->X, m->Y, n, m->st));
    CK(cudaMemcpyAsync(y, m->Y, sizeof(float) * FSI_MLP_OUT * n, cudaMemcpyDeviceToHost, m->st));
    CK(cudaStreamSynchronize(m->st));
    return FSI_OK;
}

int fsi_mlp_grad(fsi_mlp_t m, const float *x, const float *y, int n, float *grad, float *loss) {
    if (!m || n <= 0 || !x || !y || !grad) return fail(FSI_E_ARG, "invalid argument");
    if (!m->norm_set) return fail(FSI_E_STATE, "network statistics not set (fsi_mlp_set_norm)");
    if (int rc = mlp_reserve(m, n)) return rc;
    CK(cudaMemcpyAsync(m->X, x, sizeof(float) * FSI_MLP_IN * n, cudaMemcpyHostToDevice, m->st));
    CK(cudaMemcpyAsync(m->Y, y, sizeof(float) * FSI_MLP_OUT * n, cudaMemcpyHostToDevice, m->st));
    CK(cudaMemsetAsync(m->grad, 0, sizeof(float) * FSI_MLP_NPARAM, m->st));
    CK(cudaMemsetAsync(m->loss, 0, sizeof(float), m->st));
    CK(launch_mlp_grad(m->P, m->nrm, m->X, m->Y, nullptr, 0, n, n, m->grad, m->loss, m->st));
    CK(cudaMemcpyAsync(grad, m->grad, sizeof(float) * FSI_MLP_NPARAM, cudaMemcpyDeviceToHost, m->st));
    float l = 0.0f;
    CK(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
    CK(cudaMemsetAsync(m->grad, 0, sizeof(float) * FSI_MLP_NPARAM, m->st));
    CK(cudaStreamSynchronize(m->st));
    if (loss) *loss = l;
    return FSI_OK;
}

int fsi_mlp_train(fsi_mlp_t m, const float *x, const float *y, int n, int epochs, int batch, float lr,
                  unsigned long long seed, float *loss_per_epoch) {
    FSI_CALL_RANGE();
    if (!m || n <= 0 || !x || !y || epochs <= 0 || batch <= 0 || !(lr > 0.0f))
        return fail(FSI_E_ARG, "invalid argument");
    if (!m->norm_set) return fail(FSI_E_STATE, "network statistics not set (fsi_mlp_set_norm)");
    if (int rc = mlp_reserve(m, n)) return rc;
    if (epochs > m->loss_cap) {
        CK(cudaStreamSynchronize(m->st));
        cudaFree(m->loss);
        m->loss = nullptr;
        m->loss_cap = 0;
        CK(cudaMalloc((void **)&m->loss, sizeof(float) * epochs));
        m->loss_cap = epochs;
    }
    batch = std::min(batch, n);
    const int nbatch = (n + batch - 1) / batch;
    CK(cudaMemcpyAsync(m->X, x, sizeof(float) * FSI_MLP_IN * n, cudaMemcpyHostToDevice, m->st));
    CK(cudaMemcpyAsync(m->Y, y, sizeof(float) * FSI_MLP_OUT * n, cudaMemcpyHostToDevice, m->st));
    CK(cudaMemsetAsync(m->loss, 0, sizeof(float) * epochs, m->st));
    CK(cudaMemsetAsync(m->grad, 0, sizeof(float) * FSI_MLP_NPARAM, m->st));
    for (int k = 0; k < 2; k++) CK(cudaEventRecord(m->ev[k], m->st));
    // Sample orders alternate between two slots: the host refills a slot only
    // after the copy of its previous use has run (the slot's event).
    uint64_t r = seed;
    for (int e = 0; e < epochs; e++) {
        const int k = e & 1;
        int *hp = m->hperm + (long long)k * m->cap, *dp = m->perm + (long long)k * m->cap;
        CK(cudaEventSynchronize(m->ev[k]));
        for (int i = 0; i < n; i++) hp[i] = i;
        for (int i = n - 1; i > 0; i--) std::swap(hp[i], hp[(int)(splitmix64(r) % (uint64_t)(i + 1))]);
        CK(cudaMemcpyAsync(dp, hp, sizeof(int) * n, cudaMemcpyHostToDevice, m->st));
        for (int b = 0; b < nbatch; b++) {
            const int b0 = b * batch, nb = std::min(batch, n - b0);
            CK(launch_mlp_grad(m->P, m->nrm, m->X, m->Y, dp, b0, nb, nb, m->grad, m->loss + e, m->st));
            CK(launch_mlp_adam(m->P, m->grad, m->m, m->v, lr, ++m->t, m->st));
        }
        CK(cudaEventRecord(m->ev[k], m->st));
    }
    std::vector<float> hl(epochs);
    CK(cudaMemcpyAsync(hl.data(), m->loss, sizeof(float) * epochs, cudaMemcpyDeviceToHost, m->st));
    CK(cudaStreamSynchronize(m->st));
    if (loss_per_epoch)
        for (int e = 0; e < epochs; e++) loss_per_epoch[e] = hl[e] / (float)nbatch;
    return FSI_OK;
}

}  // extern "C"

// ----------------------------------------------------------- batched blocks
// Many independent blocks stepped together: per step one upload of every
// block's tables and markers, one launch of the IB stage of all blocks (one
// CTA each), one launch of the bulk step of all blocks, one of their window
// fix-ups, one per face index, and one download of every force and status;
// captured once as a CUDA graph and replayed.

struct fsi_batch {
    int n = 0;
    std::vector<fsi_block *> blk;
    int prec = 0, model = 1;
    cudaStream_t st = nullptr, st2 = nullptr;  // st2: the IB stage, beside the bulk step
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evf = nullptr, evj = nullptr;
    int threads = BATCH_THREADS[0];  // bulk kernel CTA size (the autotuner's choice; 0: per-case form)
    // the per-case form of the bulk step (threads == 0): each block's own
    // single-block bulk kernel, its arguments in the launch, fanned out over
    // streams inside the captured graph; those arguments are baked in, so
    // there is one graph per buffer parity (gexec: the buffers as captured,
    // gexec_odd: swapped) and a recapture when a block's bulk arguments change
    cudaStream_t fan[BATCH_FAN] = {};
    cudaEvent_t evfan[BATCH_FAN] = {};
    cudaEvent_t evfork = nullptr;
    cudaGraphExec_t gexec_odd = nullptr;
    int parity = 0;
    std::vector<StepArgs> cap_args;  // the blocks' bulk arguments at capture
    std::vector<int> moff;           // first packed marker of each block (n+1)
    int Mall = 0;
    int ntol_cap = 0;
    // one device region and its pinned mirror: [BatchCase n][IbCoop n][BcArgs 6n][xyz 3M][vel 3M][area M]
    size_t off_ib = 0, off_bc = 0, off_mk = 0, in_bytes = 0;
    unsigned char *d_in = nullptr, *h_in = nullptr;
    double *d_ef = nullptr, *h_ef = nullptr;  // 3M
    int *d_stat = nullptr, *h_stat = nullptr;  // 8 per block
    double *d_res = nullptr, *h_res = nullptr;  // per block
    double *d_tol = nullptr;                    // ntol_cap per block
    // block of each row group, for each CTA size (filled once)
    int *d_gcase[3] = {nullptr, nullptr, nullptr};
    int G[3] = {0, 0, 0};
    bool face_on[6] = {false, false, false, false, false, false};
    int Amax[6] = {0, 0, 0, 0, 0, 0}, Bmax[6] = {0, 0, 0, 0, 0, 0};
    cudaGraphExec_t gexec = nullptr;
    int g_threads = 0, g_ntol = 0;
    long long g_wmax = -1;
    bool g_forced = false;
};

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int thread_slot(int T) {
    for (int k = 0; k < 3; k++)
        if (BATCH_THREADS[k] == T) return k;
    return 0;
}

void free_batch(fsi_batch *b) {
    if (!b) return;
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->gexec_odd) cudaGraphExecDestroy(b->gexec_odd);
    for (int k = 0; k < BATCH_FAN; k++) {
        if (b->evfan[k]) cudaEventDestroy(b->evfan[k]);
        if (b->fan[k]) cudaStreamDestroy(b->fan[k]);
    }
    if (b->evfork) cudaEventDestroy(b->evfork);
    void *dp[] = {b->d_in, b->d_ef, b->d_stat, b->d_res, b->d_tol, b->d_gcase[0], b->d_gcase[1], b->d_gcase[2]};
    for (void *p : dp)
        if (p) cudaFree(p);
    void *hp[] = {b->h_in, b->h_ef, b->h_stat, b->h_res};
    for (void *p : hp)
        if (p) cudaFreeHost(p);
    cudaEvent_t evs[] = {b->ev0, b->ev1, b->evf, b->evj};
    for (cudaEvent_t ev : evs)
        if (ev) cudaEventDestroy(ev);
    if (b->st2) cudaStreamDestroy(b->st2);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

// row groups of every block for CTAs of T threads; returns the total
int batch_groups(fsi_batch *b, int T, BatchCase *cs) {
    int g0 = 0;
    for (int c = 0; c < b->n; c++) {
        const fsi_block *h = b->blk[c];
        const int tpr = h->Z / 2;
        const int R = std::max(1, T / tpr);
        cs[c].tpr = tpr;
        cs[c].R = R;
        cs[c].ngy = (h->Y + R - 1) / R;
        cs[c].g0 = g0;
        g0 += cs[c].ngy * h->X;
    }
    return g0;
}

// the bulk step tables of every block (fa -> fb) into the staging area
void batch_fill_steps(fsi_batch *b, const double *vf, const double *blktime, bool use_window) {
    BatchCase *cs = (BatchCase *)b->h_in;
    for (int c = 0; c < b->n; c++) {
        fsi_block *h = b->blk[c];
        fill_step(h, vf + 3 * c, blktime[c], use_window, cs[c].a);
        for (int k = 0; k < 19; k++) cs[c].sd[k] = (float)h->mm.sd[k];
    }
}

// the bulk arguments of block c for the per-case form: the bulk kernel
// alone (the window fix-up runs batched), buffers swapped for odd parity
StepArgs percase_args(const fsi_batch *b, int c, int parity) {
    StepArgs a = ((const BatchCase *)b->h_in)[c].a;
    a.win = Win{};
    a.win.x1 = a.win.x0 - 1;
    a.win.n = 0;
    a.join = nullptr;
    if (parity) {
        const void *t = a.src;
        a.src = a.dst;
        a.dst = const_cast<void *>(t);
    }
    return a;
}

// the per-case bulk kernels, fanned out from st over the fan streams and
// joined back into st (inside a capture, or for the autotuner)
cudaError_t percase_launch(fsi_batch *b, int parity) {
    const int nf = std::min(b->n, BATCH_FAN);
    cudaError_t e = cudaEventRecord(b->evfork, b->st);
    for (int k = 0; k < nf && e == cudaSuccess; k++) e = cudaStreamWaitEvent(b->fan[k], b->evfork, 0);
    for (int c = 0; c < b->n && e == cudaSuccess; c++) {
        const fsi_block *h = b->blk[c];
        e = launch_step_fast(percase_args(b, c, parity), &h->mm, b->prec, b->model, b->fan[c % nf]);
    }
    for (int k = 0; k < nf && e == cudaSuccess; k++) {
        e = cudaEventRecord(b->evfan[k], b->fan[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->evfan[k], 0);
    }
    return e;
}

// one step's graph; parity < 0: the table-driven bulk kernel
int batch_capture_one(fsi_batch *b, int G, long long wmax, bool forced, int parity, cudaGraphExec_t *out) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemcpyAsync(b->d_in, b->h_in, b->in_bytes, cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_stat, 0, sizeof(int) * 8 * b->n, b->st);
    // the IB stage (second stream) and the bulk step only read the state;
    // the window fix-up needs both
    if (e == cudaSuccess) e = cudaEventRecord(b->evf, b->st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st2, b->evf, 0);
    if (e == cudaSuccess) e = launch_batch_ib((const IbCoop *)(b->d_in + b->off_ib), b->n, 512, b->prec, b->st2);
    if (e == cudaSuccess) e = cudaEventRecord(b->evj, b->st2);
    if (e == cudaSuccess) {
        if (parity < 0)
            e = launch_batch_step((const BatchCase *)b->d_in, b->d_gcase[thread_slot(b->threads)], b->n, G, b->threads,
                                  0, b->prec, b->model, forced, b->st);
        else
            e = percase_launch(b, parity);
    }
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->evj, 0);
    if (e == cudaSuccess) e = launch_batch_winfix((const BatchCase *)b->d_in, b->n, wmax, b->prec, b->model, b->st);
    for (int k = 0; k < 6 && e == cudaSuccess; k++)
        if (b->face_on[k])
            e = launch_batch_bc((const BcArgs *)(b->d_in + b->off_bc) + (size_t)k * b->n, b->n, k, b->Amax[k],
                                b->Bmax[k], b->prec, b->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->h_ef, b->d_ef, sizeof(double) * 3 * std::max(1, b->Mall), cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->h_stat, b->d_stat, sizeof(int) * 8 * b->n, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->h_res, b->d_res, sizeof(double) * b->n, cudaMemcpyDeviceToHost, b->st);
    cudaError_t ce = cudaStreamEndCapture(b->st, &g);
    if (e != cudaSuccess) return fail(FSI_E_CUDA, "batch capture: %s", cudaGetErrorString(e));
    if (ce != cudaSuccess) return fail(FSI_E_CUDA, "batch capture: %s", cudaGetErrorString(ce));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(FSI_E_CUDA, "batch graph: %s", cudaGetErrorString(e));
    return FSI_OK;
}

int batch_capture(fsi_batch *b, int G, long long wmax, bool forced) {
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->gexec_odd) {
        cudaGraphExecDestroy(b->gexec_odd);
        b->gexec_odd = nullptr;
    }
    if (b->threads == 0) {
        int rc = batch_capture_one(b, G, wmax, forced, 0, &b->gexec);
        if (!rc) rc = batch_capture_one(b, G, wmax, forced, 1, &b->gexec_odd);
        if (rc) return rc;
        b->cap_args.resize(b->n);
        for (int c = 0; c < b->n; c++) b->cap_args[c] = ((const BatchCase *)b->h_in)[c].a;
        b->parity = 0;
    } else {
        int rc = batch_capture_one(b, G, wmax, forced, -1, &b->gexec);
        if (rc) return rc;
    }
    b->g_threads = b->threads;
    b->g_wmax = wmax;
    b->g_forced = forced;
    b->g_ntol = b->ntol_cap;
    return FSI_OK;
}

// the per-case graphs still hold this step's bulk arguments: the buffers of
// the current parity, the same volume force and z-face populations
bool percase_current(const fsi_batch *b) {
    if ((int)b->cap_args.size() != b->n) return false;
    const BatchCase *cs = (const BatchCase *)b->h_in;
    for (int c = 0; c < b->n; c++) {
        const StepArgs &x = cs[c].a, &y = b->cap_args[c];
        const bool swapped = b->parity != 0;
        if (x.src != (swapped ? (const void *)y.dst : y.src) || x.dst != (swapped ? const_cast<void *>(y.src) : y.dst))
            return false;
        for (int k = 0; k < 3; k++)
            if (x.vf[k] != y.vf[k]) return false;
        for (int k = 0; k < 2; k++) {
            if (x.zeq[k] != y.zeq[k]) return false;
            for (int q = 0; q < 19; q++)
                if (x.zg[k][q] != y.zg[k][q]) return false;
        }
    }
    return true;
}

}  // namespace

extern "C" {

int fsi_batch_create(fsi_batch_t *out, int n, const fsi_block_t *blocks) {
    if (!out || n <= 0 || !blocks) return fail(FSI_E_ARG, "invalid argument");
    *out = nullptr;
    for (int c = 0; c < n; c++) {
        fsi_block *h = blocks[c];
        if (!h) return fail(FSI_E_ARG, "block %d is null", c);
        if (h->prec != FSI_PREC_F32 && h->prec != FSI_PREC_F16 && h->prec != FSI_PREC_BF16)
            return fail(FSI_E_ARG, "block %d: batches take the offset storage forms (F32, F16, BF16)", c);
        if (h->prec != blocks[0]->prec || h->d.iCollidModel != blocks[0]->d.iCollidModel)
            return fail(FSI_E_ARG, "block %d: all blocks of a batch share the storage form and collision model", c);
        if (h->d.iCollidModel != CM_SRT && h->d.iCollidModel != CM_MRT && h->d.iCollidModel != CM_TRT &&
            h->d.iCollidModel != CM_SMAG)
            return fail(FSI_E_ARG, "block %d: batches run SRT, TRT, MRT or Smagorinsky", c);
        StepArgs a;
        double z3[3] = {0, 0, 0};
        fill_step(h, z3, 0.0, false, a);
        if (!step_fast_paired(a, &h->mm, h->prec, h->d.iCollidModel) || h->Z / 2 > 512)
            return fail(FSI_E_ARG, "block %d: needs the paired kernels (even zDim <= 1024, diagonal MRT)", c);
        if ((unsigned long long)19 * h->N * h->esz >= (1ULL << 32))
            return fail(FSI_E_ARG, "block %d: a batched block's distributions must span less than 4 GiB", c);
        for (int k = 0; k < 6; k++) {
            const int code = h->d.bndConds[k];
            if (code == BC_NEQ || code == BC_WALL_HW || code == BC_MWALL_HW || code == BC_FLUID ||
                code == BC_FLUID_FATHER)
                return fail(FSI_E_ARG, "block %d face %d: code %d is not supported in a batch", c, k, code);
        }
        for (int c2 = 0; c2 < c; c2++)
            if (blocks[c2] == h) return fail(FSI_E_ARG, "block %d appears twice", c);
    }
    fsi_batch *b = new (std::nothrow) fsi_batch;
    if (!b) return fail(FSI_E_ARG, "out of host memory");
    b->n = n;
    b->blk.assign(blocks, blocks + n);
    b->prec = blocks[0]->prec;
    b->model = blocks[0]->d.iCollidModel;
    b->moff.assign(n + 1, 0);
    for (int c = 0; c < n; c++) b->moff[c + 1] = b->moff[c] + b->blk[c]->Mtot;
    b->Mall = b->moff[n];
    for (int c = 0; c < n; c++) {
        const fsi_block *h = b->blk[c];
        for (int k = 0; k < 6; k++) {
            const int code = h->d.bndConds[k];
            if (code == BC_PERIODIC) continue;
            b->face_on[k] = true;
            const int ax = k >> 1;
            b->Amax[k] = std::max(b->Amax[k], ax < 2 ? h->Z : h->Y);
            b->Bmax[k] = std::max(b->Bmax[k], ax == 0 ? h->Y : h->X);
        }
    }
    const int Mt = std::max(1, b->Mall);
    b->off_ib = align256(sizeof(BatchCase) * n);
    b->off_bc = b->off_ib + align256(sizeof(IbCoop) * n);
    b->off_mk = b->off_bc + align256(sizeof(BcArgs) * 6 * n);
    b->in_bytes = b->off_mk + sizeof(double) * 7 * Mt;
    auto bail = [&](cudaError_t e) {
        free_batch(b);
        return fail(FSI_E_CUDA, "batch allocation: %s", cudaGetErrorString(e));
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreate(&b->ev0)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreate(&b->ev1)) != cudaSuccess) return bail(e);
    {
        int lo = 0, hi = 0;
        if ((e = cudaDeviceGetStreamPriorityRange(&lo, &hi)) != cudaSuccess) return bail(e);
        if ((e = cudaStreamCreateWithPriority(&b->st2, cudaStreamNonBlocking, hi)) != cudaSuccess) return bail(e);
    }
    if ((e = cudaEventCreateWithFlags(&b->evf, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreateWithFlags(&b->evj, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreateWithFlags(&b->evfork, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
    for (int k = 0; k < std::min(n, BATCH_FAN); k++) {
        if ((e = cudaStreamCreateWithFlags(&b->fan[k], cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
        if ((e = cudaEventCreateWithFlags(&b->evfan[k], cudaEventDisableTiming)) != cudaSuccess) return bail(e);
    }
    if ((e = cudaMalloc((void **)&b->d_in, b->in_bytes)) != cudaSuccess) return bail(e);
    if ((e = cudaHostAlloc((void **)&b->h_in, b->in_bytes, cudaHostAllocDefault)) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc((void **)&b->d_ef, sizeof(double) * 3 * Mt)) != cudaSuccess) return bail(e);
    if ((e = cudaHostAlloc((void **)&b->h_ef, sizeof(double) * 3 * Mt, cudaHostAllocDefault)) != cudaSuccess)
        return bail(e);
    if ((e = cudaMalloc((void **)&b->d_stat, sizeof(int) * 8 * n)) != cudaSuccess) return bail(e);
    if ((e = cudaHostAlloc((void **)&b->h_stat, sizeof(int) * 8 * n, cudaHostAllocDefault)) != cudaSuccess)
        return bail(e);
    if ((e = cudaMalloc((void **)&b->d_res, sizeof(double) * n)) != cudaSuccess) return bail(e);
    if ((e = cudaHostAlloc((void **)&b->h_res, sizeof(double) * n, cudaHostAllocDefault)) != cudaSuccess)
        return bail(e);
    memset(b->h_in, 0, b->in_bytes);
    // the block of every row group, for each CTA size
    for (int k = 0; k < 3; k++) {
        std::vector<BatchCase> cs(n);
        b->G[k] = batch_groups(b, BATCH_THREADS[k], cs.data());
        std::vector<int> gc(b->G[k]);
        for (int c = 0; c < n; c++)
            for (int j = cs[c].g0; j < (c + 1 < n ? cs[c + 1].g0 : b->G[k]); j++) gc[j] = c;
        if ((e = cudaMalloc((void **)&b->d_gcase[k], sizeof(int) * std::max(1, b->G[k]))) != cudaSuccess) return bail(e);
        if ((e = cudaMemcpyAsync(b->d_gcase[k], gc.data(), sizeof(int) * b->G[k], cudaMemcpyHostToDevice, b->st)) !=
            cudaSuccess)
            return bail(e);
        if ((e = cudaStreamSynchronize(b->st)) != cudaSuccess) return bail(e);
    }
    // the blocks' own queued work finishes before the batch takes them over
    for (int c = 0; c < n; c++)
        if ((e = cudaStreamSynchronize(b->blk[c]->st)) != cudaSuccess) return bail(e);
    *out = b;
    return FSI_OK;
}

int fsi_batch_destroy(fsi_batch_t b) {
    if (!b) return FSI_OK;
    cudaStreamSynchronize(b->st);
    free_batch(b);
    return FSI_OK;
}

int fsi_batch_ib_step(fsi_batch_t b, const double *xyz, const double *vel, const double *area, const double *vf,
                      const double *denIn, const double *dt, const double *Uref, int ntol, double dtol,
                      const double *blktime, double *eforce, int *iters, double *residual) {
    FSI_CALL_RANGE();
    if (!b || !vf || !denIn || !dt || !Uref || !blktime || ntol < 0) return fail(FSI_E_ARG, "null argument");
    if (b->Mall > 0 && (!xyz || !vel || !area || !eforce)) return fail(FSI_E_ARG, "null marker array");
    const int n = b->n;
    // the marker slices were laid out when the batch was made
    for (int c = 0; c < n; c++)
        if (b->blk[c]->Mtot != b->moff[c + 1] - b->moff[c])
            return fail(FSI_E_STATE, "block %d: its bodies changed after fsi_batch_create", c);
    // the penalty residual sums of every block
    if (ntol > b->ntol_cap) {
        CK(cudaStreamSynchronize(b->st));
        if (b->d_tol) cudaFree(b->d_tol);
        b->d_tol = nullptr;
        b->ntol_cap = 0;
        const int cap = std::max(ntol, 64);
        CK(cudaMalloc((void **)&b->d_tol, sizeof(double) * cap * n));
        b->ntol_cap = cap;
    }
    // windows (host, from the markers) and the tables
    long long wmax = 0;
    bool forced = false;
    BatchCase *cs = (BatchCase *)b->h_in;
    IbCoop *ib = (IbCoop *)(b->h_in + b->off_ib);
    BcArgs *bc = (BcArgs *)(b->h_in + b->off_bc);
    double *mk = (double *)(b->h_in + b->off_mk);
    double *dmk = (double *)(b->d_in + b->off_mk);
    const int Mt = std::max(1, b->Mall);
    for (int c = 0; c < n; c++) {
        fsi_block *h = b->blk[c];
        const int m0 = b->moff[c];
        h->win_valid = false;
        if (h->Mtot > 0) {
            int rc = compute_window(h, xyz + 3LL * m0);
            if (rc) return fail(rc, "block %d: %s", c, g_err.c_str());
            h->win_valid = true;
            wmax = std::max(wmax, h->Nw_cap);
        }
        for (int k = 0; k < 3; k++) forced = forced || vf[3 * c + k] != 0.0;
        fill_step(h, vf + 3 * c, blktime[c], h->Mtot > 0, cs[c].a);
        for (int k = 0; k < 19; k++) cs[c].sd[k] = (float)h->mm.sd[k];
        if (h->Mtot > 0) {
            fill_ib(h, vf + 3 * c, denIn[c], dt[c], Uref[c], ntol, dtol, ib[c]);
            ib[c].xyz = dmk + 3LL * m0;
            ib[c].vel = dmk + 3LL * Mt + 3LL * m0;
            ib[c].area = dmk + 6LL * Mt + m0;
            ib[c].eforce = b->d_ef + 3LL * m0;
            ib[c].tol_acc = b->d_tol + (size_t)b->ntol_cap * c;
            ib[c].status = b->d_stat + 8 * c;
            ib[c].res = b->d_res + c;
        } else {
            ib[c] = IbCoop{};
        }
        for (int k = 0; k < 6; k++) {
            BcArgs a;
            if (fill_bc(h, k, h->fb, blktime[c], cs[c].a.zeq, a)) bc[(size_t)k * n + c] = a;
            else {
                bc[(size_t)k * n + c] = BcArgs{};
                bc[(size_t)k * n + c].code = BC_FLUID;
            }
        }
    }
    const int G = batch_groups(b, b->threads, cs);
    if (b->Mall > 0) {
        memcpy(mk, xyz, sizeof(double) * 3 * b->Mall);
        memcpy(mk + 3LL * Mt, vel, sizeof(double) * 3 * b->Mall);
        memcpy(mk + 6LL * Mt, area, sizeof(double) * b->Mall);
    }
    if (!b->gexec || b->g_threads != b->threads || b->g_wmax < wmax || b->g_forced != forced ||
        b->g_ntol != b->ntol_cap || (b->threads == 0 && !percase_current(b))) {
        int rc = batch_capture(b, G, wmax, forced);
        if (rc) return rc;
    }
    CK(cudaGraphLaunch(b->threads == 0 && b->parity ? b->gexec_odd : b->gexec, b->st));
    CK(cudaStreamSynchronize(b->st));
    b->parity ^= 1;
    for (int c = 0; c < n; c++) {
        fsi_block *h = b->blk[c];
        std::swap(h->fa, h->fb);
        h->win_valid = false;
    }
    for (int c = 0; c < n; c++) {
        if (b->blk[c]->Mtot == 0) {
            if (iters) iters[c] = 0;
            if (residual) residual[c] = 0.0;
            continue;
        }
        const int stt = b->h_stat[8 * c];
        if (stt & 1) return fail(FSI_E_RANGE, "block %d: index out of block bounds in IB stencil", c);
        if (stt & 2) return fail(FSI_E_RANGE, "block %d: IB stencil outside the IB window", c);
        if (stt & 4) return fail(FSI_E_NAN, "block %d: Nan found in PenaltyForce", c);
        if (iters) iters[c] = b->h_stat[8 * c + 1];
        if (residual) residual[c] = b->h_res[c];
    }
    if (b->Mall > 0) memcpy(eforce, b->h_ef, sizeof(double) * 3 * b->Mall);
    return FSI_OK;
}

int fsi_batch_tune(fsi_batch_t b, int reps, int *threads, float *ms_per_step) {
    FSI_CALL_RANGE();
    if (!b || reps <= 0) return fail(FSI_E_ARG, "invalid argument");
    // the bulk step of every block, fa -> fb without swapping: the state does
    // not change (fb is rewritten by the next step)
    std::vector<double> vf(3 * b->n, 0.0), t(b->n, 0.0);
    batch_fill_steps(b, vf.data(), t.data(), false);
    BatchCase *cs = (BatchCase *)b->h_in;
    float best = 1e30f;
    int best_t = b->threads;
    for (int T : BATCH_THREADS) {
        const int G = batch_groups(b, T, cs);
        CK(cudaMemcpyAsync(b->d_in, b->h_in, b->off_ib, cudaMemcpyHostToDevice, b->st));
        const int *gc = b->d_gcase[thread_slot(T)];
        for (int w = 0; w < 2; w++)
            CK(launch_batch_step((const BatchCase *)b->d_in, gc, b->n, G, T, 0, b->prec, b->model, false, b->st));
        CK(cudaEventRecord(b->ev0, b->st));
        for (int r = 0; r < reps; r++)
            CK(launch_batch_step((const BatchCase *)b->d_in, gc, b->n, G, T, 0, b->prec, b->model, false, b->st));
        CK(cudaEventRecord(b->ev1, b->st));
        CK(cudaEventSynchronize(b->ev1));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        ms /= (float)reps;
        if (ms < best) {
            best = ms;
            best_t = T;
        }
    }
    // the per-case form: a graph of the blocks' own bulk kernels, fanned out
    {
        cudaGraph_t g;
        cudaGraphExec_t ge = nullptr;
        CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = percase_launch(b, 0);
        cudaError_t ce = cudaStreamEndCapture(b->st, &g);
        if (e != cudaSuccess || ce != cudaSuccess)
            return fail(FSI_E_CUDA, "batch tune capture: %s", cudaGetErrorString(e != cudaSuccess ? e : ce));
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(FSI_E_CUDA, "batch tune graph: %s", cudaGetErrorString(e));
        for (int w = 0; w < 2 && e == cudaSuccess; w++) e = cudaGraphLaunch(ge, b->st);
        if (e == cudaSuccess) e = cudaEventRecord(b->ev0, b->st);
        for (int r = 0; r < reps && e == cudaSuccess; r++) e = cudaGraphLaunch(ge, b->st);
        if (e == cudaSuccess) e = cudaEventRecord(b->ev1, b->st);
        if (e == cudaSuccess) e = cudaEventSynchronize(b->ev1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        cudaGraphExecDestroy(ge);
        if (e != cudaSuccess) return fail(FSI_E_CUDA, "batch tune: %s", cudaGetErrorString(e));
        ms /= (float)reps;
        if (ms < best) {
            best = ms;
            best_t = 0;
        }
    }
    b->threads = best_t;
    if (threads) *threads = best_t;
    if (ms_per_step) *ms_per_step = best;
    return FSI_OK;
}

int fsi_batch_set_threads(fsi_batch_t b, int threads) {
    if (!b) return fail(FSI_E_ARG, "null handle");
    if (threads == 0) {
        b->threads = 0;
        return FSI_OK;
    }
    for (int T : BATCH_THREADS)
        if (T == threads) {
            b->threads = threads;
            return FSI_OK;
        }
    return fail(FSI_E_ARG, "unsupported CTA size %d", threads);
}

}  // extern "C"

// ------------------------------------------------- allocation-free variant
// Scratch of fsi_pair_father_to_son_static: the interpolated son face
// (19 populations per face cell) followed by its interpolated tau, for at
// most FSI_STATIC_FACE_CELLS face cells. A device holds this array from the
// first fsi_pair_create on it (which looks up its address) until the process
// exits.
static __device__ __align__(256) double g_pair_face_scratch[20LL * FSI_STATIC_FACE_CELLS];

namespace {
std::mutex g_scratch_mu;
double *g_scratch_ptr[256] = {};  // device address of the array, per device

// looked up once per device, with that device current (fsi_pair_create
// does it, so the static calls that follow find it resolved)
int static_scratch(double **out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return fail(FSI_E_ARG, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_pair_face_scratch);
        if (e != cudaSuccess) return fail(FSI_E_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return FSI_OK;
}
}  // namespace

extern "C" int fsi_pair_father_to_son_static(fsi_pair_t p, int n_timeStep, const double vf[3]) {
    FSI_CALL_RANGE();
    if (!p || !vf) return fail(FSI_E_ARG, "invalid argument");
    fsi_block *so = p->so, *fa = p->fa;
    for (int k = 0; k < 6; k++) {
        if (p->p.sds[k] == 0) continue;
        int ax = k >> 1;
        long long AS = ax == 2 ? p->p.yDimS : p->p.zDimS, BS = ax == 0 ? p->p.yDimS : p->p.xDimS;
        if (AS * BS > FSI_STATIC_FACE_CELLS)
            return fail(FSI_E_ARG, "son face of %lld cells exceeds the static scratch of %d face cells", AS * BS,
                        FSI_STATIC_FACE_CELLS);
    }
    double *scr = nullptr;
    int rc = static_scratch(&scr);
    if (rc) return rc;
    double *scr_f = scr, *scr_t = scr + 19LL * FSI_STATIC_FACE_CELLS;
    CK(cudaStreamSynchronize(fa->st));
    for (int k = 0; k < 6; k++) {
        if (p->p.sds[k] == 0) continue;
        int lvl = (n_timeStep == 0) ? 0 : 1;
        CK(launch_pair_f2s(so->fa, so->prec, so->X, so->Y, so->Z, tau_src(so), p->p, k, p->buf[k][lvl], p->buft[k][lvl],
                           p->scheme, scr_f, scr_t, FSI_STATIC_FACE_CELLS, vf, fa->d.dh, p->d_err, so->st));
    }
    CK(cudaStreamSynchronize(so->st));
    return pair_check(p);
}
