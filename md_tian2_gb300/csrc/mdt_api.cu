// mdt_api.cu -- the C ABI (include/mdt_gpu.h): context, batch layout, transfers and
// launch orchestration.  No torch types; plain pointers and sizes only.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/mdt_gpu.h"
#include "mdt_common.cuh"
#include "mdt_internal.h"

using namespace mdt;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct mdt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int64_t launches = 0;
    int num_sms = 0;

    // PES
    bool have_emt = false;
    EmtConst E{};
    int pes_ntypes = 0;

    // batch
    bool have_batch = false;
    // refill: state of the last upload (6 SoA arrays), generation per trajectory, counter
    double *tmpl = nullptr;
    int *gen = nullptr, *refill_count = nullptr;
    double *draws = nullptr;  // per trajectory the last refill's draws (u, w, einc, polar, azimuth)
    bool have_tmpl = false;
    int step_limit = 0;
    double ads_start = kDefaultReal, ads_end = kDefaultReal;  // adsorption hysteresis (A)
    int T = 0, ntypes = 0, max_atoms = 0, max_beads = 0;
    int64_t total_ba = 0, total_pairs = 0;
    int total_atoms = 0, total_beads = 0;
    std::vector<int> natoms, nbeads, atom_off, bead_off;
    std::vector<int> h_type;  // universe type per atom (host copy)
    std::vector<int64_t> ba_off;
    Batch B{};
    std::vector<DevBuf> bufs;
    double *stage = nullptr;   // 13 * total_ba doubles: one Fortran-order slice per array of a transfer
    int *order = nullptr, *counter = nullptr, *ba_traj = nullptr;
    double *rnd[4] = {nullptr, nullptr, nullptr, nullptr};
    double *summary = nullptr;
    size_t scratch_prec_bytes = 0;

    // HDNNP / surrogate
    bool have_nn = false;
    NNDev M{};
    int ngeta_max = 0;
    std::vector<void *> nnbufs;  // model arrays (live across batches)
    int pes_kind = MDT_PES_EMT;
    double margin = 0.1;
    NNScratch X{};
    int nn_maxnb_alloc = 0;
    // FP32 fast path (mdt_nnf.cu): tables, host copies of the scaling data, switch
    FastNN F{};
    bool fast_enabled = true;
    std::vector<double> h_smin, h_smax, h_savg;
    float4 *d_scal = nullptr;
    float *d_dscal = nullptr;
    unsigned *mscr = nullptr;  // fast-path mask scratch (grows on demand)
    size_t mscr_n = 0;
    // fast-path Verlet skin lists (with the batch); skin in A (0: off)
    int2 *skw = nullptr;
    int *skcnt = nullptr, *skok = nullptr;
    double *skref = nullptr;
    int skcap = 0;
    double skin_ang = 1.0;
    bool skin_dirty = true;
    int sk_layout = -1;        // 0: warp-per-atom lists, 1: thread-per-atom lists (entry-major)
    // thread-per-atom kernel of radial-only models (mdt_nnr.cu): tables, switch, pack plan
    RadialNN R{};
    bool radial_enabled = true;
    int2 *rpacks = nullptr;    // (offset into rptraj, count) per pack
    int *rptraj = nullptr;     // trajectories of the packs
    int rnpack = 0, rblock = 0;
    bool rfull = false;         // the plan packs every trajectory of the batch (not a re-pack)
    double *lcoef = nullptr;    // constant-friction Langevin coefficients of the thread-per-atom kernel
    RadialNN RG{};              // tensor-core network tables of a generic model (own descriptor order)
    double *tc_G = nullptr;     // its pass buffers: raw descriptors, atomic energies [ba][maxsf], [ba]
    double *tc_eat = nullptr;
    float *tc_dg = nullptr;     // dE/dG [ba][maxsf]
    // BF16 GEMM training (mdt_train_gemm.cu): cuBLAS handle, row list, pools, per-slot buffers
    cublasHandle_t cublas = nullptr;
    int *g_slot = nullptr;
    int g_cap = 0;              // rows the pools hold
    float *g_f = nullptr, *g_gw = nullptr;
    __nv_bfloat16 *g_b = nullptr;
    float *g_dg = nullptr, *g_xdot = nullptr;
    double *g_eat = nullptr, *g_arow = nullptr;
    double lc_key[4] = {0, 0, 0, 0};  // (gamma, step, Tsurf, Tproj) they were formed for
    bool lc_valid = false;
    int rmaxblock = kRBlockMax; // largest block the pack plan may use
    int *tcerr = nullptr;       // device word: a tensor-core GEMM of the network timed out

    // training (buffers live with the batch)
    bool have_labels = false;
    double *t_E = nullptr, *t_fx = nullptr, *t_fy = nullptr, *t_fz = nullptr, *t_G = nullptr;
    double *t_grad = nullptr, *t_loss = nullptr;
    float *t_theta = nullptr, *t_m = nullptr, *t_v = nullptr;
    int *t_conf = nullptr;
    int t_step = 0;
};

namespace {

const char *const kBf16Scope =
    "MDT_PREC_BF16 / MDT_PREC_BF16X3 run the network GEMMs on the tensor cores: fused MD steps and forces of a "
    "radial-only network in the thread-per-atom kernel (single-bead trajectories of at most 512 atoms), and "
    "mdt_calc_force of an MDT_PES_NENE model whose network has at most two elements, two hidden layers of <= 32 "
    "nodes with one activation (p t s l) per layer and <= 48 descriptors";

int fail(mdt_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(mdt_ctx *c, cudaError_t e, const char *where) {
    return fail(c, MDT_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename T> T *dalloc(mdt_ctx *c, size_t n, cudaError_t &e) {
    void *p = nullptr;
    const size_t bytes = std::max<size_t>(n * sizeof(T), 16);
    e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return nullptr;
    c->bufs.push_back(DevBuf{p, bytes});
    return (T *)p;
}

void free_batch(mdt_ctx *c) {
    c->X = NNScratch{};
    c->tmpl = nullptr;
    c->gen = c->refill_count = nullptr;
    c->draws = nullptr;
    c->have_tmpl = false;
    c->skw = nullptr;
    c->skcnt = c->skok = nullptr;
    c->skref = nullptr;
    c->skcap = 0;
    c->skin_dirty = true;
    c->sk_layout = -1;
    c->rpacks = nullptr;
    c->rptraj = nullptr;
    c->rnpack = c->rblock = 0;
    c->lcoef = nullptr;
    c->lc_valid = false;
    c->tc_G = c->tc_eat = nullptr;
    c->tc_dg = nullptr;
    c->g_slot = nullptr;
    c->g_cap = 0;
    c->g_f = c->g_gw = nullptr;
    c->g_b = nullptr;
    c->g_dg = c->g_xdot = nullptr;
    c->g_eat = c->g_arow = nullptr;
    c->have_labels = false;
    c->nn_maxnb_alloc = 0;
    for (auto &b : c->bufs) cudaFree(b.p);
    c->bufs.clear();
    c->have_batch = false;
    c->stage = nullptr;
    c->order = c->counter = c->ba_traj = nullptr;
    for (auto &r : c->rnd) r = nullptr;
    c->summary = nullptr;
}

// cjk normal-mode matrix, src/rpmd.f90:36-59 (column major, j 1-based in the arguments)
void build_cjk(int nb, double *c) {
    const double pi = kPi;
    for (int j = 1; j <= nb; ++j)
        for (int k = 0; k <= nb - 1; ++k) {
            double v;
            if (k == 0) v = std::sqrt(1.0 / nb);
            else if (1 <= k && k <= nb / 2 - 1) v = std::sqrt(2.0 / nb) * std::cos(2.0 * pi * j * k / nb);
            else if (k == nb / 2) v = std::sqrt(1.0 / nb) * ((j % 2) ? -1.0 : 1.0);
            else v = std::sqrt(2.0 / nb) * std::sin(2.0 * pi * j * k / nb);
            c[(size_t)k * nb + (j - 1)] = v;
        }
}

// invert_matrix, src/useful_things.f90:296-321 (column major)
bool invert3(const double *A, double *B) {
    auto a = [&](int i, int j) { return A[(j - 1) * 3 + (i - 1)]; };
    const double det = a(1, 1) * a(2, 2) * a(3, 3) - a(1, 1) * a(2, 3) * a(3, 2) - a(1, 2) * a(2, 1) * a(3, 3) +
                       a(1, 2) * a(2, 3) * a(3, 1) + a(1, 3) * a(2, 1) * a(3, 2) - a(1, 3) * a(2, 2) * a(3, 1);
    if (det < kTolerance) return false;
    const double di = 1 / det;
    auto b = [&](int i, int j) -> double & { return B[(j - 1) * 3 + (i - 1)]; };
    b(1, 1) = +di * (a(2, 2) * a(3, 3) - a(2, 3) * a(3, 2));
    b(2, 1) = -di * (a(2, 1) * a(3, 3) - a(2, 3) * a(3, 1));
    b(3, 1) = +di * (a(2, 1) * a(3, 2) - a(2, 2) * a(3, 1));
    b(1, 2) = -di * (a(1, 2) * a(3, 3) - a(1, 3) * a(3, 2));
    b(2, 2) = +di * (a(1, 1) * a(3, 3) - a(1, 3) * a(3, 1));
    b(3, 2) = -di * (a(1, 1) * a(3, 2) - a(1, 2) * a(3, 1));
    b(1, 3) = +di * (a(1, 2) * a(2, 3) - a(1, 3) * a(2, 2));
    b(2, 3) = -di * (a(1, 1) * a(2, 3) - a(1, 3) * a(2, 1));
    b(3, 3) = +di * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1));
    return true;
}

PropParams to_dev(const mdt_ctx *c, const mdt_prop_params *p) {
    PropParams P{};
    P.step = p->step;
    P.Tsurf = p->Tsurf;
    P.Tproj = p->Tproj;
    P.pile_tau = p->pile_tau;
    P.andersen_time = p->andersen_time;
    P.gamma_const = p->gamma_const;
    P.pul = p->pul;
    P.pll = p->pll;
    P.seed = p->seed;
    P.use_exit = p->use_exit;
    P.rng_mode = p->rng_mode;
    P.max_steps = c->step_limit;
    P.ads_start = c->ads_start;
    P.ads_end = c->ads_end;
    P.randy = c->rnd[0];
    P.zeta = c->rnd[1];
    P.andersen_v = c->rnd[2];
    P.andersen_u = c->rnd[3];
    return P;
}

int check_ready(mdt_ctx *c, bool need_emt) {
    if (!c) return MDT_ERR_ARG;
    if (!c->have_batch) return fail(c, MDT_ERR_STATE, "no batch defined (call mdt_batch_define)");
    if (need_emt && !c->have_emt) return fail(c, MDT_ERR_STATE, "no PES parameters (call mdt_emt_set_params)");
    if (need_emt && c->pes_ntypes != c->ntypes)
        return fail(c, MDT_ERR_ARG, "PES and batch disagree on the number of types");
    return MDT_OK;
}

LaunchCfg cfg(mdt_ctx *c, int precision) {
    const int per_sm = max_resident_ctas(c->max_atoms, c->max_beads, precision);
    const int grid = std::max(1, std::min(c->T, c->num_sms * per_sm));
    return LaunchCfg{c->stream, grid, c->order, c->counter};
}

int ensure_scratch(mdt_ctx *c, int precision) {
    const size_t rs = precision == MDT_PREC_FP32 ? 4 : 8;
    const size_t need = std::max<size_t>(16, 6 * rs * (size_t)c->total_pairs);
    if (c->B.pair_scratch && c->scratch_prec_bytes >= need) return MDT_OK;
    cudaError_t e;
    void *p = dalloc<unsigned char>(c, need, e);
    if (!p) return fail(c, MDT_ERR_NOMEM, "pair scratch allocation failed");
    c->B.pair_scratch = p;
    c->scratch_prec_bytes = need;
    return MDT_OK;
}


// image counts of neighbor_para_short.f90:59-108 for one cell (columns in A)
void image_counts(const double *box, double cutoff_bohr, int *out) {
    const double a2b = 1.0 / kBohr2Ang;
    auto L = [&](int i, int k) { return box[3 * (i - 1) + (k - 1)] * a2b; };
    double axb[3] = {L(1, 2) * L(2, 3) - L(1, 3) * L(2, 2), L(1, 3) * L(2, 1) - L(1, 1) * L(2, 3),
                     L(1, 1) * L(2, 2) - L(1, 2) * L(2, 1)};
    double axc[3] = {L(1, 2) * L(3, 3) - L(1, 3) * L(3, 2), L(1, 3) * L(3, 1) - L(1, 1) * L(3, 3),
                     L(1, 1) * L(3, 2) - L(1, 2) * L(3, 1)};
    double bxc[3] = {L(2, 2) * L(3, 3) - L(2, 3) * L(3, 2), L(2, 3) * L(3, 1) - L(2, 1) * L(3, 3),
                     L(2, 1) * L(3, 2) - L(2, 2) * L(3, 1)};
    auto nrm = [](double *v) {
        const double a = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        v[0] /= a; v[1] /= a; v[2] /= a;
    };
    nrm(axb); nrm(axc); nrm(bxc);
    const double pa = std::fabs(L(1, 1) * bxc[0] + L(1, 2) * bxc[1] + L(1, 3) * bxc[2]);
    const double pb = std::fabs(L(2, 1) * axc[0] + L(2, 2) * axc[1] + L(2, 3) * axc[2]);
    const double pc = std::fabs(L(3, 1) * axb[0] + L(3, 2) * axb[1] + L(3, 3) * axb[2]);
    int na = 0, nb = 0, nc = 0;
    while ((double)na * pa <= cutoff_bohr) ++na;
    while ((double)nb * pb <= cutoff_bohr) ++nb;
    while ((double)nc * pc <= cutoff_bohr) ++nc;
    out[0] = na; out[1] = nb; out[2] = nc;
}

int ensure_nn_scratch(mdt_ctx *c) {
    if (c->X.nbw && c->nn_maxnb_alloc == c->M.maxnb) return MDT_OK;
    cudaError_t e = cudaSuccess;
    int *nbw = dalloc<int>(c, (size_t)c->total_ba * c->M.maxnb, e);
    int *nbcnt = dalloc<int>(c, (size_t)c->total_ba, e);
    int *img = dalloc<int>(c, 3 * (size_t)c->T, e);
    int *fb = dalloc<int>(c, (size_t)c->T, e);
    int *st = dalloc<int>(c, (size_t)c->T, e);
    if (!nbw || !nbcnt || !img || !fb || !st) return fail(c, MDT_ERR_NOMEM, "neighbour-list scratch allocation failed");
    std::vector<int> h(3 * (size_t)c->T);
    std::vector<double> box(9 * (size_t)c->T);
    e = cudaMemcpy(box.data(), c->B.box, sizeof(double) * box.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "cell download");
    for (int t = 0; t < c->T; ++t) {
        image_counts(box.data() + 9 * t, c->M.maxcut, h.data() + 3 * t);
        for (int k = 0; k < 3; ++k)
            if (h[3 * t + k] > 7) return fail(c, MDT_ERR_UNSUPPORTED, "cell too small for the cutoff (more than 7 images)");
    }
    if (c->max_atoms > 65535) return fail(c, MDT_ERR_UNSUPPORTED, "more than 65535 atoms");
    e = cudaMemcpyAsync(img, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(fb, 0, sizeof(int) * c->T, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(st, 0, sizeof(int) * c->T, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(nbcnt, 0, sizeof(int) * c->total_ba, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "neighbour-list scratch set-up");
    c->X = NNScratch{nbw, nbcnt, img, fb, st};
    c->nn_maxnb_alloc = c->M.maxnb;
    return MDT_OK;
}

LaunchCfg nn_cfg(mdt_ctx *c, int precision) {
    const int per_sm = nn_resident_ctas(c->M, c->max_atoms, c->max_beads, c->ngeta_max, precision,
                                        c->pes_kind == MDT_PES_SURROGATE);
    const int grid = std::max(1, std::min(c->T, c->num_sms * per_sm));
    return LaunchCfg{c->stream, grid, c->order, c->counter};
}

// Scaling of the fast path in FP32: scaled = x g + y, range flag outside [z, w], and the
// factor RuNNer applies to dG/dx (getshortatomic.f90:174-236).
int upload_fast_scaling(mdt_ctx *c) {
    if (!c->F.ok || !c->d_scal) return MDT_OK;
    const NNDev &M = c->M;
    const size_t n = (size_t)M.nelem * M.maxsf;
    std::vector<float4> sc(n, make_float4(1.f, 0.f, -INFINITY, INFINITY));
    std::vector<float> ds(n, 1.f);
    for (int e = 0; e < M.nelem; ++e)
        for (int s = 0; s < M.nsf[e]; ++s) {
            const size_t k = (size_t)e * M.maxsf + s;
            const double mn = c->h_smin[k], mx = c->h_smax[k], avg = c->h_savg[k], w = mx - mn;
            double a = 1.0, b = 0.0;
            if (M.centersym && !M.scalesym) b = -avg;
            else if (M.scalesym && !M.centersym) { a = (M.scmax - M.scmin) / w; b = M.scmin - mn * a; }
            else if (M.scalesym && M.centersym) { a = 1.0 / w; b = -avg / w; }
            sc[k] = make_float4((float)a, (float)b, (float)(mn - c->margin * w), (float)(mx + c->margin * w));
            ds[k] = M.scalesym ? (float)((M.scmax - M.scmin) / w) : 1.f;
        }
    cudaError_t e = cudaMemcpy(c->d_scal, sc.data(), sizeof(float4) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_dscal, ds.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "fast-path scaling upload");
}

// FastNN tables of a model (FastNN::ok = 0 when it does not qualify).
FastNN build_fast(const NNDev &M, const mdt_nn_model *m, const std::vector<int> &e1, const std::vector<int> &etaslot,
                  std::vector<float4> &g2tab) {
    FastNN F{};
    g2tab.assign((size_t)kMaxElem * kFMaxG2, make_float4(0.f, 0.f, 0.f, 0.f));
    F.ok = 0;
    if (M.cutoff_type != 1 || M.cutoff_alpha != 0.0 || M.maxnb > 255) return F;
    const int ms = M.maxsf;
    int zm = 0, ng = 1;
    for (int e = 0; e < M.nelem; ++e) {
        if (M.rc[e] != M.maxcut) return F;
        int n2 = 0, n3 = 0;
        for (int s = 0; s < M.nsf[e]; ++s) {
            const int k = e * ms + s;
            if (m->sftype[k] == 2) {
                ++n2;
                continue;
            }
            ++n3;
            const double z = m->zeta[k];
            int b = -1;
            for (int t = 0; t < 5; ++t)
                if (z == (double)(1 << t)) b = t;
            if (b < 0 || (m->lambda[k] != 1.0 && m->lambda[k] != -1.0)) return F;
            zm |= 1 << b;
        }
        if (n2 > kFMaxG2 || (n3 > 0 && !M.g3fast[e]) || M.ng3eta[e] > 4) return F;
        ng = std::max(ng, M.ng3eta[e]);
    }
    const int zs = nnf_zm_supported(zm);
    if (!zs) return F;
    F.zm = zs;
    F.ng = ng;
    int bit_index[5], nz = 0;
    for (int b = 0; b < 5; ++b) bit_index[b] = (zs >> b) & 1 ? nz++ : -1;
    for (int b = 0; b < 5; ++b)
        if (bit_index[b] >= 0) {
            F.cell_lz[2 * bit_index[b]] = (float)(1 << b);
            F.cell_lz[2 * bit_index[b] + 1] = -(float)(1 << b);
        }
    const double rc = M.maxcut;
    F.rc2 = (float)(rc * rc);
    F.inv_rc2 = (float)(1.0 / (rc * rc));
    const double cut2 = rc * rc;
    F.cut2_hi = (float)cut2 * 1.0001f;
    F.cut2_lo = (float)cut2 * 0.9999f;
    const double log2e = 1.4426950408889634;
    for (int e = 0; e < M.nelem; ++e) {
        for (int a = 0; a < 4; ++a)
            for (int q = 0; q < kFNQ; ++q) F.cell_sf[e][a][q] = -1;
        for (int a = 0; a < 4; ++a) {
            F.g3eta[e][a] = a < M.ng3eta[e] ? (float)M.g3eta[e][a] : 0.f;
            F.g3l2[e][a] = a < M.ng3eta[e] ? (float)(-M.g3eta[e][a] * log2e) : 0.f;
        }
        F.hasg3[e] = 0;
        F.pair_a[e] = F.pair_b[e] = -1;
        F.ng2[e] = 0;
        for (int s = 0; s < M.nsf[e]; ++s) {
            const int k = e * ms + s;
            if (m->sftype[k] == 2) {
                ++F.ng2[e];
                continue;
            }
            int b = 0;
            while ((double)(1 << b) != m->zeta[k]) ++b;
            const int q = 2 * bit_index[b] + (m->lambda[k] < 0.0 ? 1 : 0);
            F.cell_sf[e][etaslot[k]][q] = (int8_t)s;
            F.hasg3[e] = 1;
            F.pair_a[e] = M.g3pair[e][0];
            F.pair_b[e] = M.g3pair[e][1];
        }
    }
    // radial functions grouped by neighbour element, ascending eta (then r_s)
    for (int e = 0; e < M.nelem; ++e) {
        int pos = 0;
        for (int a = 0; a < M.nelem; ++a) {
            std::vector<int> idx;
            for (int s = 0; s < M.nsf[e]; ++s) {
                const int k = e * ms + s;
                if (m->sftype[k] == 2 && e1[k] == a) idx.push_back(s);
            }
            std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) {
                const double ex = m->eta[e * ms + x], ey = m->eta[e * ms + y];
                return ex != ey ? ex < ey : m->rshift[e * ms + x] < m->rshift[e * ms + y];
            });
            for (int s : idx) {
                const int k = e * ms + s;
                float4 v = make_float4((float)(-m->eta[k] * log2e), (float)m->rshift[k], (float)(-2.0 * m->eta[k]), 0.f);
                const int bits = s | (a << 8);
                std::memcpy(&v.w, &bits, 4);
                g2tab[e * kFMaxG2 + pos++] = v;
            }
        }
    }
    F.anyg3 = 0;
    for (int e = 0; e < M.nelem; ++e) F.anyg3 |= F.hasg3[e];
    // shared-memory weight layout: rows padded to a stride = 4 (mod 8) floats
    int off = 0;
    for (int e = 0; e < M.nelem; ++e)
        for (int l = 1; l <= M.nlayers; ++l) {
            int str = (M.nodes[e][l] + 3) & ~3;
            if (str % 8 == 0) str += 4;
            F.wstr[e][l] = str;
            F.wofs[e][l] = off;
            off += (M.nodes[e][l - 1] + 1) * str;
        }
    F.wtotal = off;
    F.ok = 1;
    return F;
}

// RadialNN tables of a model (RadialNN::ok = 0 when it does not qualify; see mdt_nn.cuh).
RadialNN build_radial(const NNDev &M, const mdt_nn_model *m, const FastNN &F, const std::vector<int> &e1) {
    RadialNN R{};
    R.ok = 0;
    if (!F.ok || F.anyg3 || M.nelem > 2 || (M.nlayers != 2 && M.nlayers != 3)) return R;
    const int ne = M.nelem, ms = M.maxsf, nh = M.nlayers - 1;
    for (int e = 0; e < ne; ++e) {
        for (int l = 1; l <= nh; ++l)
            if (M.nodes[e][l] > 32) return R;
        if (M.nodes[e][M.nlayers] != 1) return R;
        if (M.normnodes)
            for (int l = 0; l <= M.nlayers; ++l)
                if (M.nodes[e][l] != M.nodes[0][l]) return R;
    }
    // one activation per layer over nodes and elements, of the kinds the kernel has
    for (int l = 0; l < M.nlayers; ++l) {
        const uint8_t a = m->act[((size_t)0 * m->nlayers + l) * m->maxnodes];
        if (!std::strchr("ptsl", (int)a) || a == 0) return R;
        for (int e = 0; e < ne; ++e)
            for (int n = 0; n < M.nodes[e][l + 1]; ++n)
                if (m->act[((size_t)e * m->nlayers + l) * m->maxnodes + n] != a) return R;
        R.act[l] = a;
        R.rn[l] = M.normnodes ? (float)(1.0 / M.nodes[0][l]) : 1.f;
    }
    // (eta, r_s) list per neighbour element, identical for every centre element
    std::vector<int> idx[kMaxElem][2];
    for (int e = 0; e < ne; ++e)
        for (int g = 0; g < 2; ++g) {
            for (int s = 0; s < M.nsf[e]; ++s)
                if (m->sftype[e * ms + s] == 2 && e1[e * ms + s] == g) idx[e][g].push_back(s);
            std::stable_sort(idx[e][g].begin(), idx[e][g].end(), [&](int x, int y) {
                const double ex = m->eta[e * ms + x], ey = m->eta[e * ms + y];
                return ex != ey ? ex < ey : m->rshift[e * ms + x] < m->rshift[e * ms + y];
            });
        }
    for (int e = 0; e < ne; ++e) {
        int n2 = 0;
        for (int s = 0; s < M.nsf[e]; ++s) n2 += m->sftype[e * ms + s] == 2 && (e1[e * ms + s] == 0 || e1[e * ms + s] == 1);
        if (n2 != M.nsf[e]) return R;  // every function over an element of the model
        for (int g = 0; g < 2; ++g) {
            if (idx[e][g].size() != idx[0][g].size() || idx[e][g].size() > (size_t)kRMaxK) return R;
            for (size_t k = 0; k < idx[e][g].size(); ++k) {
                const int a = e * ms + idx[e][g][k], b = idx[0][g][k];
                if (m->eta[a] != m->eta[b] || m->rshift[a] != m->rshift[b]) return R;
            }
        }
    }
    const int cnt0 = (int)idx[0][0].size(), cnt1 = (int)idx[0][1].size();
    // recurrence admission per neighbour group: one eta, r_s evenly spaced (within 1e-9
    // bohr), and blocks short enough that a block start below the FP32 range (2^-126,
    // flushed to zero) hides only functions below 2^-40: (L - 1) delta <= 4.9 / sqrt(|c|)
    // with c = -eta log2(e) (sqrt(126) - sqrt(40) = 4.9)
    int maxbl[2] = {0, 0};
    double dl[2] = {0.0, 0.0};
    for (int g = 0; g < 2; ++g) {
        const std::vector<int> &v = idx[0][g];
        if (v.size() < 2) continue;
        const double eta0 = m->eta[v[0]];
        const double d = (m->rshift[v.back()] - m->rshift[v[0]]) / (double)(v.size() - 1);
        bool uni = eta0 > 0.0 && d > 0.0;
        for (size_t k = 0; k < v.size() && uni; ++k) {
            uni = m->eta[v[k]] == eta0 && std::fabs(m->rshift[v[k]] - (m->rshift[v[0]] + d * (double)k)) <= 1e-9;
        }
        if (!uni) continue;
        const double c = eta0 * 1.4426950408889634;
        maxbl[g] = 1 + (int)std::floor(4.9 / std::sqrt(c) / d);
        dl[g] = d;
    }
    if (!nnr_shape(cnt0, cnt1, nh, maxbl, R)) return R;
    const int ka = R.ka, kb = R.kb;
    for (int g = 0; g < 2; ++g) {
        const double c = -m->eta[idx[0][g].empty() ? 0 : idx[0][g][0]] * 1.4426950408889634;
        R.dl[g] = (float)dl[g];
        R.gq[g] = (float)(-2.0 * c * dl[g]);
        R.gc[g] = (float)(c * dl[g] * dl[g]);
        R.gam[g] = (float)std::exp2(2.0 * c * dl[g] * dl[g]);
    }
    R.nh = nh;
    R.nelem = ne;
    R.nin = ka + kb;
    const double log2e = 1.4426950408889634;
    for (int g = 0; g < 2; ++g)
        for (int k = 0; k < kRMaxK; ++k) {
            const bool on = k < (int)idx[0][g].size();
            R.c[g][k] = on ? (float)(-m->eta[idx[0][g][k]] * log2e) : 0.f;
            R.rs[g][k] = on ? (float)m->rshift[idx[0][g][k]] : 0.f;
        }
    for (int e = 0; e < 2; ++e)
        for (int q = 0; q < 2 * kRMaxK; ++q) R.qsrc[e][q] = -1;
    for (int e = 0; e < ne; ++e) {
        for (int k = 0; k < cnt0; ++k) R.qsrc[e][k] = (int8_t)idx[e][0][k];
        for (int k = 0; k < cnt1; ++k) R.qsrc[e][ka + k] = (int8_t)idx[e][1][k];
    }
    const double rc = M.maxcut;
    R.rc2 = (float)(rc * rc);
    R.inv_rc2 = (float)(1.0 / (rc * rc));
    R.rc_b = (float)rc;
    R.maxnb = M.maxnb;
    for (int t = 0; t < kMaxTypes; ++t) R.elem_of_type[t] = M.elem_of_type[t];
    for (int e = 0; e < 2; ++e) R.atom_energy[e] = e < ne ? M.atom_energy[e] : 0.0;
    R.maxweights = M.maxweights;
    R.maxsf = M.maxsf;
    for (int e = 0; e < 2; ++e)
        for (int l = 0; l <= kMaxLayers; ++l) {
            R.woff[e][l] = e < ne && l <= M.nlayers ? M.woff[e][l] : 0;
            R.nodes[e][l] = e < ne && l <= M.nlayers ? M.nodes[e][l] : 0;
        }
    R.ok = 1;
    return R;
}

// Tensor-core network tables of a model that does not run on the thread-per-atom kernel (any
// descriptors, e.g. with G3): the network of build_radial's form -- at most two elements, one or
// two hidden layers of <= 32 nodes, one activation per layer of the kinds p t s l, one output
// node -- on at most 48 descriptors in the model's own order; the descriptors' scaling comes
// from the fast path's table (FastNN::scal, dscal).  RadialNN::ok = 0 otherwise.
RadialNN build_tc_generic(const NNDev &M, const mdt_nn_model *m, const FastNN &F) {
    RadialNN R{};
    R.ok = 0;
    if (!F.ok || M.nelem > 2 || (M.nlayers != 2 && M.nlayers != 3)) return R;
    const int ne = M.nelem, nh = M.nlayers - 1;
    int nsf = 0;
    for (int e = 0; e < ne; ++e) {
        nsf = std::max(nsf, M.nsf[e]);
        for (int l = 1; l <= nh; ++l)
            if (M.nodes[e][l] > 32) return R;
        if (M.nodes[e][M.nlayers] != 1) return R;
        if (M.normnodes)
            for (int l = 0; l <= M.nlayers; ++l)
                if (M.nodes[e][l] != M.nodes[0][l]) return R;
    }
    if (nsf > 48) return R;
    for (int l = 0; l < M.nlayers; ++l) {
        const uint8_t a = m->act[((size_t)0 * m->nlayers + l) * m->maxnodes];
        if (!std::strchr("ptsl", (int)a) || a == 0) return R;
        for (int e = 0; e < ne; ++e)
            for (int n = 0; n < M.nodes[e][l + 1]; ++n)
                if (m->act[((size_t)e * m->nlayers + l) * m->maxnodes + n] != a) return R;
        R.act[l] = a;
        R.rn[l] = M.normnodes ? (float)(1.0 / M.nodes[0][l]) : 1.f;
    }
    R.nh = nh;
    R.nelem = ne;
    R.nin = nsf <= 24 ? 24 : 48;
    for (int e = 0; e < 2; ++e)
        for (int q = 0; q < 2 * kRMaxK; ++q) R.qsrc[e][q] = (int8_t)(e < ne && q < M.nsf[e] ? q : -1);
    for (int t = 0; t < kMaxTypes; ++t) R.elem_of_type[t] = M.elem_of_type[t];
    for (int e = 0; e < 2; ++e) R.atom_energy[e] = e < ne ? M.atom_energy[e] : 0.0;
    R.maxweights = M.maxweights;
    R.maxsf = M.maxsf;
    for (int e = 0; e < 2; ++e)
        for (int l = 0; l <= kMaxLayers; ++l) {
            R.woff[e][l] = e < ne && l <= M.nlayers ? M.woff[e][l] : 0;
            R.nodes[e][l] = e < ne && l <= M.nlayers ? M.nodes[e][l] : 0;
        }
    R.ok = 1;
    return R;
}

bool use_fast(mdt_ctx *c, int precision) {
    if (precision != MDT_PREC_FP32 || !c->F.ok || !c->fast_enabled) return false;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return nnf_total_smem(c->B, c->M, c->F) <= (size_t)optin;
}

LaunchCfg nnf_cfg(mdt_ctx *c) {
    const int per_sm = nnf_resident_ctas(c->B, c->M, c->F);
    const int grid = std::max(1, std::min(c->T, c->num_sms * per_sm));
    return LaunchCfg{c->stream, grid, c->order, c->counter};
}

int ensure_mscr(mdt_ctx *c, int grid, int layout);

// Pack plan of the thread-per-atom kernel for the batch.  A pack is a set of whole
// trajectories run by one CTA (thread = atom).  For w waves of the resident CTAs the
// trajectories are dealt largest first to the pack with the fewest atoms (at most
// kRMaxTraj per pack); the block is the largest pack rounded up to a warp, and the
// smallest w whose block fits the cap wins (one CTA per SM is resident, so the largest
// CTAs keep the most warps in flight; the latency-bound kernel gains more from them than
// it loses to the emptier last wave).
// ids: the trajectories to pack (all of them when empty); a re-pack over the trajectories
// still running drops the threads of stopped ones (mdt_nn_repack)
bool radial_plan(mdt_ctx *c, const std::vector<int> &ids = {}) {
    if (c->rnpack > 0 && ids.empty()) return true;
    if (c->max_beads != 1 || c->max_atoms > kRBlockMax) return false;
    for (int t = 0; t < c->ntypes; ++t)
        if (c->R.elem_of_type[t] < 0) return false;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (nnr_smem(c->R) > (size_t)optin ||
        nnr_emt_smem(c->max_atoms) > 4 * (size_t)nnr_hbw(c->R.nin, c->R.nh) * kRBlockMax)
        return false;
    // the kernel's image loops span at most 65 cells per direction: every cell must be wider
    // than the skin-list cutoff / 32 in each direction
    {
        std::vector<double> box(9 * (size_t)c->T);
        if (cudaMemcpy(box.data(), c->B.box, sizeof(double) * box.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
            return false;
        const double rcs = c->M.maxcut * kBohr2Ang + c->skin_ang;  // A
        for (int t = 0; t < c->T; ++t) {
            const double *a = box.data() + 9 * (size_t)t;  // cell vectors a[0..2], a[3..5], a[6..8]
            auto cross = [&](int p, int q, double *o) {
                o[0] = a[3 * p + 1] * a[3 * q + 2] - a[3 * p + 2] * a[3 * q + 1];
                o[1] = a[3 * p + 2] * a[3 * q] - a[3 * p] * a[3 * q + 2];
                o[2] = a[3 * p] * a[3 * q + 1] - a[3 * p + 1] * a[3 * q];
            };
            double x[3];
            cross(1, 2, x);
            const double vol = std::fabs(a[0] * x[0] + a[1] * x[1] + a[2] * x[2]);
            for (int d = 0; d < 3; ++d) {
                cross((d + 1) % 3, (d + 2) % 3, x);
                const double area = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
                if (!(vol > 0.0) || !(area > 0.0) || !(32.0 * vol / area > rcs)) return false;
            }
        }
    }
    c->R.block = kRBlockMax;
    const int slots = c->num_sms * std::max(1, nnr_resident_ctas(c->R));
    std::vector<int> order(ids.empty() ? c->T : (int)ids.size());
    if (ids.empty()) std::iota(order.begin(), order.end(), 0);
    else std::copy(ids.begin(), ids.end(), order.begin());
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return c->natoms[a] > c->natoms[b]; });
    int64_t total = 0;
    for (int t : order) total += c->natoms[t];
    const int ntr = (int)order.size();
    if (ntr == 0) return c->rnpack > 0;
    const int bmax = std::max(32, std::min(kRBlockMax, c->rmaxblock));
    if (c->max_atoms > bmax) return false;
    const int w0 = (int)std::max<int64_t>(1, (total + (int64_t)slots * bmax - 1) / ((int64_t)slots * bmax));
    std::vector<std::vector<int>> bestp;
    int bestb = 0;
    for (int w = w0; w <= w0 + 4; ++w) {
        const int np = std::min<int64_t>((int64_t)w * slots, ntr);
        std::vector<std::vector<int>> packs(np);
        std::vector<int> load(np, 0);
        // min-heap of (atoms, pack) over packs that still take trajectories
        std::vector<std::pair<int, int>> heap;
        for (int k = 0; k < np; ++k) heap.emplace_back(0, k);
        auto cmp = [](const std::pair<int, int> &a, const std::pair<int, int> &b) { return a > b; };
        std::make_heap(heap.begin(), heap.end(), cmp);
        bool ok = true;
        for (int t : order) {
            if (heap.empty()) {
                ok = false;
                break;
            }
            std::pop_heap(heap.begin(), heap.end(), cmp);
            const int k = heap.back().second;
            heap.pop_back();
            packs[k].push_back(t);
            load[k] += c->natoms[t];
            if ((int)packs[k].size() < kRMaxTraj) {
                heap.emplace_back(load[k], k);
                std::push_heap(heap.begin(), heap.end(), cmp);
            }
        }
        if (!ok) continue;
        const int mx = *std::max_element(load.begin(), load.end());
        const int block = (mx + 31) & ~31;
        if (block > bmax) continue;
        // fewest waves first: the largest CTAs keep the most warps per SM in flight
        bestp = std::move(packs);
        bestb = block;
        break;
    }
    if (bestp.empty()) return false;
    // packs largest first (the work queue hands them out in order)
    std::stable_sort(bestp.begin(), bestp.end(), [&](const std::vector<int> &a, const std::vector<int> &b) {
        int la = 0, lb = 0;
        for (int t : a) la += c->natoms[t];
        for (int t : b) lb += c->natoms[t];
        return la > lb;
    });
    std::vector<int2> hp;
    std::vector<int> ht;
    for (auto &p : bestp) {
        if (p.empty()) continue;
        std::sort(p.begin(), p.end());
        hp.push_back(make_int2((int)ht.size(), (int)p.size()));
        ht.insert(ht.end(), p.begin(), p.end());
    }
    // the plan's buffers hold one pack and one entry per trajectory of the batch: every plan,
    // of all trajectories or of those still running, fits
    cudaError_t e = cudaSuccess;
    if (!c->rpacks) c->rpacks = dalloc<int2>(c, (size_t)c->T, e);
    if (!c->rptraj) c->rptraj = dalloc<int>(c, (size_t)c->T, e);
    if (!c->rpacks || !c->rptraj) return false;
    if (cudaMemcpyAsync(c->rpacks, hp.data(), sizeof(int2) * hp.size(), cudaMemcpyHostToDevice, c->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(c->rptraj, ht.data(), sizeof(int) * ht.size(), cudaMemcpyHostToDevice, c->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return false;
    c->rnpack = (int)hp.size();
    c->rblock = bestb;
    c->rfull = ntr == c->T;
    return true;
}

// The thread-per-atom kernel runs FP32 forces of an admitted model; the fused MD step also
// needs single-bead trajectories with Verlet or constant-friction Langevin propagators.
bool use_radial(mdt_ctx *c, int precision, bool md) {
    if ((precision != MDT_PREC_FP32 && precision != MDT_PREC_BF16 && precision != MDT_PREC_BF16X3) || !c->R.ok ||
        !c->radial_enabled ||
        !c->fast_enabled)
        return false;
    if (md)
        for (int t = 0; t < c->ntypes; ++t)
            if (c->B.algo[t] != kPropVerlet && c->B.algo[t] != kPropLangevinConst) return false;
    return radial_plan(c);
}

// tcm: network on CUDA cores (0), tensor cores with BF16 operands (1), split BF16 operands (2)
int tc_mode(int precision) { return precision == MDT_PREC_BF16 ? 1 : precision == MDT_PREC_BF16X3 ? 2 : 0; }

int run_radial(mdt_ctx *c, const PropParams &P, int nsteps, int mode, bool surr, int tcm) {
    RadialNN &R = c->R;
    R.block = c->rblock;
    R.tc = tcm;
    const bool tc = tcm != 0;
    if (tc) {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (nnr_smem(R) > (size_t)optin || nnr_emt_smem(c->max_atoms) > nnr_hb_bytes(R))
            return fail(c, MDT_ERR_UNSUPPORTED, "BF16 network: trajectories too large for the kernel's shared memory");
        if (!c->tcerr) {
            cudaError_t e = cudaMalloc(&c->tcerr, sizeof(int));
            if (e == cudaSuccess) e = cudaMemsetAsync(c->tcerr, 0, sizeof(int), c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "tensor-core status word");
        }
    }
    c->X.tcerr = c->tcerr;
    const int per_sm = std::max(1, nnr_resident_ctas(R));
    const int grid = std::max(1, std::min(c->rnpack, c->num_sms * per_sm));
    int rc = ensure_mscr(c, grid, 1);
    if (rc) return rc;
    R.skin = c->F.skin;
    R.cut2s = c->F.cut2s;
    R.rcs = (float)(c->M.maxcut + c->skin_ang / kBohr2Ang);
    R.surrogate = surr ? 1 : 0;
    R.fscal = c->F.scal;
    R.fdscal = c->F.dscal;
    if (mode == 2) {
        // constant-friction coefficients depend on (gamma, dt, T) and the batch's masses and
        // propagators (fixed by mdt_batch_define): formed once per parameter set
        const double key[4] = {P.gamma_const, P.step, P.Tsurf, P.Tproj};
        if (!c->lcoef || !c->lc_valid || std::memcmp(key, c->lc_key, sizeof(key)) != 0) {
            cudaError_t e = cudaSuccess;
            if (!c->lcoef) c->lcoef = dalloc<double>(c, 8 * (size_t)c->total_ba, e);
            if (!c->lcoef) return fail(c, MDT_ERR_NOMEM, "Langevin coefficient buffer");
            e = launch_nnr_lcoef(c->stream, c->B, P, c->ba_traj, c->total_ba, c->lcoef);
            c->launches++;
            if (e != cudaSuccess) return cuda_fail(c, e, "Langevin coefficients");
            std::memcpy(c->lc_key, key, sizeof(key));
            c->lc_valid = true;
        }
    }
    c->X.lcoef = c->lcoef;
    const cudaError_t e = launch_nnr(LaunchCfg{c->stream, grid, c->order, c->counter}, c->B, R, c->E, c->X, P,
                                     c->rpacks, c->rptraj, c->rnpack, nsteps, mode);
    c->launches++;
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "network kernel (thread per atom)");
}

// mask scratch of the fast path: the triplet masks of one bead per CTA (maxnb rows of
// mw words per atom), written by the descriptor phase and read by the force phase
int ensure_mscr(mdt_ctx *c, int grid, int layout) {
    const int mw = (c->M.maxnb + 31) / 32;
    const size_t per = c->F.anyg3 ? (size_t)c->max_atoms * c->M.maxnb * mw : 4;
    const size_t n = (size_t)grid * per;
    if (n > c->mscr_n) {
        if (c->mscr) cudaFree(c->mscr);
        c->mscr = nullptr;
        c->mscr_n = 0;
        cudaError_t e = cudaMalloc(&c->mscr, n * sizeof(unsigned));
        if (e != cudaSuccess) return cuda_fail(c, e, "fast-path mask scratch");
        c->mscr_n = n;
    }
    c->X.mscr = c->mscr;
    c->X.mcap = (int)per;
    // skin lists: 2 maxnb entries per bead-atom (the skin adds about 55 % to the list)
    const int skcap = 2 * c->M.maxnb;
    cudaError_t e = cudaSuccess;
    if (!c->skw || c->skcap != skcap) {
        c->skw = dalloc<int2>(c, (size_t)c->total_ba * skcap, e);
        c->skcnt = dalloc<int>(c, (size_t)c->total_ba, e);
        c->skref = dalloc<double>(c, 3 * (size_t)c->total_ba, e);
        c->skok = dalloc<int>(c, (size_t)c->total_beads, e);
        if (!c->skw || !c->skcnt || !c->skref || !c->skok) return fail(c, MDT_ERR_NOMEM, "skin-list allocation failed");
        c->skcap = skcap;
        c->skin_dirty = true;
    }
    if (c->skin_dirty || c->sk_layout != layout) {
        e = cudaMemsetAsync(c->skok, 0, sizeof(int) * c->total_beads, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "skin-list reset");
        c->skin_dirty = false;
        c->sk_layout = layout;
    }
    c->X.skw = c->skw;
    c->X.skcnt = c->skcnt;
    c->X.skref = c->skref;
    c->X.skok = c->skok;
    c->X.skcap = skcap;
    c->F.skin = (float)(c->skin_ang / kBohr2Ang);
    const double rs = c->M.maxcut + c->skin_ang / kBohr2Ang;
    c->F.cut2s = (float)(rs * rs) * 1.0001f;
    return MDT_OK;
}

int check_nn_ready(mdt_ctx *c) {
    if (!c->have_nn) return fail(c, MDT_ERR_STATE, "no network installed (call mdt_nn_set_model)");
    if (c->pes_kind == MDT_PES_SURROGATE && !c->have_emt)
        return fail(c, MDT_ERR_STATE, "the surrogate needs EMT parameters for its fallback");
    for (int t = 0; t < c->ntypes; ++t)
        if (c->B.algo[t] == MDT_PROP_LANGEVIN)
            return fail(c, MDT_ERR_UNSUPPORTED,
                        "ldfa friction needs the EMT density (md_algo.f90:533-536); use MDT_PES_EMT");
    return ensure_nn_scratch(c);
}
}  // namespace

extern "C" {

int32_t mdt_create(int32_t device, mdt_ctx **out) {
    if (!out) return MDT_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return MDT_ERR_CUDA;
    auto *c = new mdt_ctx();
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        delete c;
        return MDT_ERR_CUDA;
    }
    c->own_stream = true;
    *out = c;
    return MDT_OK;
}

int32_t mdt_destroy(mdt_ctx *c) {
    if (!c) return MDT_ERR_ARG;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_batch(c);
    for (void *p : c->nnbufs) cudaFree(p);
    if (c->mscr) cudaFree(c->mscr);
    if (c->tcerr) cudaFree(c->tcerr);
    if (c->cublas) cublasDestroy(c->cublas);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return MDT_OK;
}

const char *mdt_last_error(const mdt_ctx *c) { return c ? c->err.c_str() : "null context"; }

int64_t mdt_launch_count(const mdt_ctx *c) { return c ? c->launches : -1; }

int32_t mdt_synchronize(mdt_ctx *c) {
    if (!c) return MDT_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_synchronize");
    if (c->tcerr) {
        int h = 0;
        e = cudaMemcpy(&h, c->tcerr, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(c, e, "mdt_synchronize");
        if (h) return fail(c, MDT_ERR_CUDA, "a tensor-core GEMM of the network did not complete within its wait limit");
    }
    return MDT_OK;
}

int32_t mdt_set_stream(mdt_ctx *c, void *s) {
    if (!c) return MDT_ERR_ARG;
    if (c->own_stream && c->stream) {
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
    }
    if (s) {
        c->stream = (cudaStream_t)s;
        c->own_stream = false;
    } else {
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        c->own_stream = true;
    }
    return MDT_OK;
}

// read_emt's parameters and the derived constants of compute_emt_1species /
// compute_emt_2species (src/pes_emt_mod.f90:258-307 and 521-592)
int32_t mdt_emt_set_params(mdt_ctx *c, int32_t ntypes, const double *eta2, const double *n0, const double *e0,
                           const double *lambda, const double *v0, const double *kappa, const double *s0,
                           const int32_t *pes) {
    if (!c) return MDT_ERR_ARG;
    if (ntypes < 1 || ntypes > kMaxTypes || !eta2 || !n0 || !e0 || !lambda || !v0 || !kappa || !s0 || !pes)
        return fail(c, MDT_ERR_ARG, "mdt_emt_set_params: bad arguments (1 <= ntypes <= 4)");
    EmtConst E{};
    const int rc = emt_derive_constants(ntypes, eta2, n0, e0, lambda, v0, kappa, s0, pes, E);
    if (rc == MDT_ERR_UNSUPPORTED) return fail(c, rc, "more than two EMT species (compute_emt_nspecies)");
    if (rc != MDT_OK) return fail(c, rc, "no EMT species in the pes table");
    c->E = E;
    c->have_emt = true;
    c->pes_ntypes = ntypes;
    return MDT_OK;
}

int32_t mdt_batch_define(mdt_ctx *c, int32_t ntraj, const int32_t *natoms, const int32_t *nbeads,
                         const int32_t *idx, const double *mass, const uint8_t *is_fixed, const double *simbox,
                         int32_t ntypes, const int32_t *algo, const uint8_t *is_proj) {
    if (!c) return MDT_ERR_ARG;
    if (ntraj < 1 || !natoms || !nbeads || !idx || !mass || !is_fixed || !simbox || !algo || !is_proj ||
        ntypes < 1 || ntypes > kMaxTypes)
        return fail(c, MDT_ERR_ARG, "mdt_batch_define: bad arguments");
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_batch(c);
    c->T = ntraj;
    c->ntypes = ntypes;
    c->natoms.assign(natoms, natoms + ntraj);
    c->nbeads.assign(nbeads, nbeads + ntraj);
    c->ba_off.resize(ntraj);
    c->atom_off.resize(ntraj);
    c->bead_off.resize(ntraj);
    std::vector<int64_t> pair_off(ntraj);
    std::vector<int> cjk_off(ntraj, 0);
    std::vector<int> nb_tables;  // distinct bead counts
    std::vector<double> cjk_host;
    int64_t ba = 0, pairs = 0;
    int at = 0, bd = 0;
    c->max_atoms = 0;
    c->max_beads = 0;
    for (int t = 0; t < ntraj; ++t) {
        const int N = natoms[t], nb = nbeads[t];
        if (N < 1 || nb < 1 || nb > 32)
            return fail(c, MDT_ERR_ARG, "natoms must be >= 1 and 1 <= nbeads <= 32");
        c->ba_off[t] = ba;
        c->atom_off[t] = at;
        c->bead_off[t] = bd;
        pair_off[t] = pairs;
        ba += (int64_t)N * nb;
        at += N;
        bd += nb;
        pairs += (int64_t)nb * N * (N / 2);
        c->max_atoms = std::max(c->max_atoms, N);
        c->max_beads = std::max(c->max_beads, nb);
        auto it = std::find(nb_tables.begin(), nb_tables.end(), nb);
        if (it == nb_tables.end()) {
            nb_tables.push_back(nb);
            const size_t off = cjk_host.size();
            cjk_host.resize(off + (size_t)nb * nb);
            build_cjk(nb, cjk_host.data() + off);
        }
    }
    {
        // offsets of each trajectory's cjk table
        std::vector<int> table_off(nb_tables.size());
        int o = 0;
        for (size_t k = 0; k < nb_tables.size(); ++k) {
            table_off[k] = o;
            o += nb_tables[k] * nb_tables[k];
        }
        for (int t = 0; t < ntraj; ++t) {
            const size_t k = std::find(nb_tables.begin(), nb_tables.end(), nbeads[t]) - nb_tables.begin();
            cjk_off[t] = table_off[k];
        }
    }
    c->total_ba = ba;
    c->total_atoms = at;
    c->total_beads = bd;
    c->total_pairs = pairs;
    if (c->max_atoms > 4096) return fail(c, MDT_ERR_UNSUPPORTED, "more than 4096 atoms in one trajectory");
    for (int a = 0; a < at; ++a)
        if (idx[a] < 1 || idx[a] > ntypes) return fail(c, MDT_ERR_ARG, "atom type index out of range");

    // host-side derived arrays
    std::vector<int8_t> type(at);
    for (int a = 0; a < at; ++a) type[a] = (int8_t)(idx[a] - 1);
    c->h_type.assign(type.begin(), type.end());
    std::vector<uint8_t> fixed(ba);
    std::vector<int> ba_traj(ba);
    for (int t = 0; t < ntraj; ++t) {
        const int N = natoms[t], nb = nbeads[t];
        for (int i = 0; i < N; ++i)
            for (int b = 0; b < nb; ++b) {
                const int64_t f = (c->ba_off[t] + (int64_t)i * nb + b) * 3;
                const int64_t s = c->ba_off[t] + (int64_t)b * N + i;
                fixed[s] = (uint8_t)((is_fixed[f] ? 1 : 0) | (is_fixed[f + 1] ? 2 : 0) | (is_fixed[f + 2] ? 4 : 0));
                ba_traj[s] = t;
            }
    }
    std::vector<double> ibox(9 * (size_t)ntraj);
    for (int t = 0; t < ntraj; ++t)
        if (!invert3(simbox + 9 * t, ibox.data() + 9 * t))
            return fail(c, MDT_ERR_ARG, "simulation cell is singular (invert_matrix)");
    std::vector<int> order(ntraj);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const double ca = (double)nbeads[a] * natoms[a] * natoms[a], cb = (double)nbeads[b] * natoms[b] * natoms[b];
        return ca > cb;
    });

    cudaError_t e = cudaSuccess;
    Batch &B = c->B;
    B = Batch{};
    B.ntraj = ntraj;
    B.ntypes = ntypes;
    B.max_atoms = c->max_atoms;
    B.max_beads = c->max_beads;
    for (int t = 0; t < kMaxTypes; ++t) {
        B.algo[t] = t < ntypes ? algo[t] : 0;
        B.is_proj[t] = t < ntypes ? (is_proj[t] ? 1 : 0) : 0;
    }
    for (int t = 0; t < ntypes; ++t)
        if (algo[t] != MDT_PROP_VERLET && algo[t] != MDT_PROP_LANGEVIN && algo[t] != MDT_PROP_ANDERSEN &&
            algo[t] != MDT_PROP_PILE && algo[t] != MDT_PROP_LANGEVIN_CONST)
            return fail(c, MDT_ERR_ARG, "unknown propagation algorithm");
#define ALLOC(ptr, T_, n)                                                          \
    do {                                                                           \
        ptr = dalloc<T_>(c, (n), e);                                               \
        if (!ptr) {                                                                \
            free_batch(c);                                                         \
            return fail(c, MDT_ERR_NOMEM, "device allocation failed: " #ptr);      \
        }                                                                          \
    } while (0)
    int *d_natoms, *d_nbeads, *d_atom_off, *d_bead_off, *d_cjk_off, *d_status, *d_steps;
    int64_t *d_ba_off, *d_pair_off;
    double *d_mass, *d_box, *d_ibox, *d_cjk;
    int8_t *d_type;
    uint8_t *d_fixed;
    ALLOC(d_natoms, int, ntraj);
    ALLOC(d_nbeads, int, ntraj);
    ALLOC(d_atom_off, int, ntraj);
    ALLOC(d_bead_off, int, ntraj);
    ALLOC(d_cjk_off, int, ntraj);
    ALLOC(d_status, int, ntraj);
    ALLOC(d_steps, int, ntraj);
    int *d_obs_i;
    double *d_obs_d;
    ALLOC(d_obs_i, int, (3 + kObsInts) * (size_t)ntraj);
    ALLOC(d_obs_d, double, (4 + kObsDots) * (size_t)ntraj);
    ALLOC(d_ba_off, int64_t, ntraj);
    ALLOC(d_pair_off, int64_t, ntraj);
    ALLOC(d_mass, double, at);
    ALLOC(d_box, double, 9 * (size_t)ntraj);
    ALLOC(d_ibox, double, 9 * (size_t)ntraj);
    ALLOC(d_cjk, double, cjk_host.size());
    ALLOC(d_type, int8_t, at);
    ALLOC(d_fixed, uint8_t, ba);
    double *arr[12];
    for (int k = 0; k < 12; ++k) ALLOC(arr[k], double, ba);
    ALLOC(B.dens, double, ba);
    ALLOC(B.epot, double, bd);
    ALLOC(c->stage, double, 13 * (size_t)ba);
    ALLOC(c->order, int, ntraj);
    ALLOC(c->counter, int, 4);
    ALLOC(c->ba_traj, int, ba);
    ALLOC(c->summary, double, 5 * (size_t)ntraj);
#undef ALLOC
    auto up = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
    };
    up(d_natoms, natoms, sizeof(int) * ntraj);
    up(d_nbeads, nbeads, sizeof(int) * ntraj);
    up(d_atom_off, c->atom_off.data(), sizeof(int) * ntraj);
    up(d_bead_off, c->bead_off.data(), sizeof(int) * ntraj);
    up(d_cjk_off, cjk_off.data(), sizeof(int) * ntraj);
    up(d_ba_off, c->ba_off.data(), sizeof(int64_t) * ntraj);
    up(d_pair_off, pair_off.data(), sizeof(int64_t) * ntraj);
    up(d_mass, mass, sizeof(double) * at);
    up(d_box, simbox, sizeof(double) * 9 * ntraj);
    up(d_ibox, ibox.data(), sizeof(double) * 9 * ntraj);
    up(d_cjk, cjk_host.data(), sizeof(double) * cjk_host.size());
    up(d_type, type.data(), at);
    up(d_fixed, fixed.data(), ba);
    up(c->order, order.data(), sizeof(int) * ntraj);
    up(c->ba_traj, ba_traj.data(), sizeof(int) * ba);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(int) * ntraj, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_steps, 0, sizeof(int) * ntraj, c->stream);
    for (int k = 0; k < 12 && e == cudaSuccess; ++k) e = cudaMemsetAsync(arr[k], 0, sizeof(double) * ba, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.dens, 0, sizeof(double) * ba, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.epot, 0, sizeof(double) * bd, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);  // host vectors go out of scope
    if (e != cudaSuccess) {
        free_batch(c);
        return cuda_fail(c, e, "mdt_batch_define upload");
    }
    B.natoms = d_natoms;
    B.nbeads = d_nbeads;
    B.ba_off = d_ba_off;
    B.atom_off = d_atom_off;
    B.bead_off = d_bead_off;
    B.pair_off = d_pair_off;
    B.rx = arr[0]; B.ry = arr[1]; B.rz = arr[2];
    B.vx = arr[3]; B.vy = arr[4]; B.vz = arr[5];
    B.ax = arr[6]; B.ay = arr[7]; B.az = arr[8];
    B.fx = arr[9]; B.fy = arr[10]; B.fz = arr[11];
    B.mass = d_mass;
    B.type = d_type;
    B.fixed = d_fixed;
    B.box = d_box;
    B.ibox = d_ibox;
    B.status = d_status;
    B.steps_done = d_steps;
    B.obs_turn = d_obs_i;
    B.obs_up = d_obs_i + ntraj;
    B.obs_clstep = d_obs_i + 2 * (size_t)ntraj;
    B.obs_cl = d_obs_d;
    B.obs_low = d_obs_d + ntraj;
    B.obs_bnc = d_obs_i + 3 * (size_t)ntraj;
    B.obs_dot = d_obs_d + 4 * (size_t)ntraj;
    B.cjk_off = d_cjk_off;
    B.cjk = d_cjk;
    B.pair_scratch = nullptr;
    c->scratch_prec_bytes = 0;
    e = launch_obs_reset(c->stream, B);
    if (e == cudaSuccess) {
        c->tmpl = dalloc<double>(c, 6 * (size_t)ba, e);
        if (e == cudaSuccess) c->gen = dalloc<int>(c, (size_t)ntraj + 1, e);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->gen, 0, sizeof(int) * ((size_t)ntraj + 1), c->stream);
        c->refill_count = c->gen ? c->gen + ntraj : nullptr;
        if (e == cudaSuccess) c->draws = dalloc<double>(c, 5 * (size_t)ntraj, e);
    }
    if (e != cudaSuccess) {
        free_batch(c);
        return cuda_fail(c, e, "mdt_batch_define observables");
    }
    c->have_batch = true;
    return MDT_OK;
}

int32_t mdt_state_upload(mdt_ctx *c, const double *r, const double *v) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    cudaError_t e = cudaSuccess;
    const size_t bytes = sizeof(double) * 3 * (size_t)c->total_ba;
    Batch &B = c->B;
    // both arrays into their own stage slices, the copies back to back; one kernel unpacks
    // them and writes the state, uploaded or kept, as the template of mdt_refill
    double *sr = r ? c->stage : nullptr, *sv = v ? c->stage + 3 * (size_t)c->total_ba : nullptr;
    if (r) e = cudaMemcpyAsync(sr, r, bytes, cudaMemcpyHostToDevice, c->stream);
    if (v && e == cudaSuccess) e = cudaMemcpyAsync(sv, v, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        e = launch_unpack_state(c->stream, B, sr, sv, c->tmpl, c->total_ba, c->ba_traj);
        c->launches++;
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(B.status, 0, sizeof(int) * c->T, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.steps_done, 0, sizeof(int) * c->T, c->stream);
    if (e == cudaSuccess) e = launch_obs_reset(c->stream, B);
    // every trajectory runs again: a re-pack over the running ones gives way to a plan of all of
    // them (a plan of all trajectories stays: the cells did not change, and the skin lists
    // check every atom's displacement since their build, whatever moved it)
    if (!c->rfull) c->rnpack = 0;
    if (e == cudaSuccess && r && v) c->have_tmpl = true;
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_state_upload");
}

int32_t mdt_state_download(mdt_ctx *c, double *r, double *v, double *f, double *a, double *epot, double *dens) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    cudaError_t e = cudaSuccess;
    const size_t bytes = sizeof(double) * 3 * (size_t)c->total_ba;
    Batch &B = c->B;
    double *outs[4] = {r, v, f, a};
    // every array packs into its own slice of the stage in one kernel; the copies then run
    // back to back and one synchronisation ends the call
    double *sl[4];
    for (int k = 0; k < 4; ++k) sl[k] = outs[k] ? c->stage + 3 * (size_t)k * c->total_ba : nullptr;
    if (r || v || f || a) {
        e = launch_pack_state(c->stream, B, sl[0], sl[1], sl[2], sl[3], c->total_ba, c->ba_traj);
        c->launches++;
    }
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
        if (outs[k]) e = cudaMemcpyAsync(outs[k], sl[k], bytes, cudaMemcpyDeviceToHost, c->stream);
    if (dens && e == cudaSuccess) {
        double *sd = c->stage + 12 * (size_t)c->total_ba;
        e = launch_pack_scalar(c->stream, B, sd, B.dens, c->total_ba, c->ba_traj);
        c->launches++;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dens, sd, sizeof(double) * c->total_ba, cudaMemcpyDeviceToHost, c->stream);
    }
    if (epot && e == cudaSuccess)
        e = cudaMemcpyAsync(epot, B.epot, sizeof(double) * c->total_beads, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_state_download");
}

int32_t mdt_set_random_arrays(mdt_ctx *c, const double *randy, const double *zeta, const double *andersen_v,
                              const double *andersen_u) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    const double *src[4] = {randy, zeta, andersen_v, andersen_u};
    const size_t n[4] = {3 * (size_t)c->total_ba, 3 * (size_t)c->total_ba, 3 * (size_t)c->total_ba,
                         (size_t)c->total_ba};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
        if (!src[k]) continue;
        if (!c->rnd[k]) {
            c->rnd[k] = dalloc<double>(c, n[k], e);
            if (!c->rnd[k]) return fail(c, MDT_ERR_NOMEM, "random array allocation failed");
        }
        e = cudaMemcpyAsync(c->rnd[k], src[k], sizeof(double) * n[k], cudaMemcpyHostToDevice, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_set_random_arrays");
}

static int check_params(mdt_ctx *c, const mdt_prop_params *p, bool draws = true) {
    if (!p) return fail(c, MDT_ERR_ARG, "null mdt_prop_params");
    if (!(p->step > 0)) return fail(c, MDT_ERR_ARG, "step must be > 0");
    if (draws && p->rng_mode == 1) {
        bool need_l = false, need_p = false, need_a = false;
        for (int t = 0; t < c->ntypes; ++t) {
            need_l |= c->B.algo[t] == MDT_PROP_LANGEVIN || c->B.algo[t] == MDT_PROP_LANGEVIN_CONST;
            need_p |= c->B.algo[t] == MDT_PROP_PILE;
            need_a |= c->B.algo[t] == MDT_PROP_ANDERSEN;
        }
        if ((need_l && !c->rnd[0]) || (need_p && !c->rnd[1]) || (need_a && (!c->rnd[2] || !c->rnd[3])))
            return fail(c, MDT_ERR_STATE, "rng_mode 1 needs mdt_set_random_arrays first");
    }
    return MDT_OK;
}

// calc_force of a generic model with its network on the tensor cores, in three passes: the
// generic FP32 kernel exports the raw descriptors (energy-only), the network runs on every
// bead-atom as 128-row tiles (launch_nn_tc), and the generic FP32 kernel forms the forces from
// the network's dE/dG by the descriptor VJP.  MDT_PES_NENE only (the surrogate's EMT fallback
// needs its range test in the same pass).
int run_tc_generic(mdt_ctx *c, const PropParams &P, int mode, int tcm) {
    if (c->pes_kind != MDT_PES_NENE || !c->RG.ok)
        return fail(c, MDT_ERR_UNSUPPORTED, kBf16Scope);
    cudaError_t e = cudaSuccess;
    const size_t nsl = (size_t)c->total_ba * c->M.maxsf;
    if (!c->tc_G) c->tc_G = dalloc<double>(c, nsl, e);
    if (!c->tc_dg) c->tc_dg = dalloc<float>(c, nsl, e);
    if (!c->tc_eat) c->tc_eat = dalloc<double>(c, (size_t)c->total_ba, e);
    if (!c->tc_G || !c->tc_dg || !c->tc_eat) return fail(c, MDT_ERR_NOMEM, "tensor-core network buffers");
    if (!c->tcerr) {
        e = cudaMalloc(&c->tcerr, sizeof(int));
        if (e == cudaSuccess) e = cudaMemsetAsync(c->tcerr, 0, sizeof(int), c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "tensor-core status word");
    }
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    RadialNN R = c->RG;
    R.tc = tcm;
    if (nn_tc_smem(R.nin, R.nh, tcm) > (size_t)optin) return fail(c, MDT_ERR_UNSUPPORTED, kBf16Scope);
    const LaunchCfg g = nn_cfg(c, MDT_PREC_FP32);
    NNScratch X = c->X;
    X.gout = c->tc_G;
    e = launch_nn(g, c->B, c->M, c->E, X, P, c->ngeta_max, 0, 1, MDT_PREC_FP32, false);  // descriptors
    c->launches++;
    const int64_t tiles = ((int64_t)c->total_ba + kRBlockMax - 1) / kRBlockMax;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, c->num_sms));
    if (e == cudaSuccess)
        e = launch_nn_tc(c->stream, grid, c->B, R, c->tc_G, c->ba_traj, c->total_ba, c->tc_dg, c->tc_eat, c->tcerr,
                         mode == 0 ? 1 : 0);
    c->launches++;
    X.gout = nullptr;
    X.dgin = c->tc_dg;
    X.eatin = c->tc_eat;
    if (e == cudaSuccess) e = launch_nn(g, c->B, c->M, c->E, X, P, c->ngeta_max, 0, mode, MDT_PREC_FP32, false);
    c->launches++;
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_calc_force (tensor-core network)");
}

int32_t mdt_calc_force(mdt_ctx *c, int32_t flag, int32_t precision, const mdt_prop_params *p) {
    int rc = check_ready(c, c && c->pes_kind == MDT_PES_EMT);
    if (rc) return rc;
    if (flag != MDT_ENERGY_AND_FORCE && flag != MDT_ENERGY_ONLY) return fail(c, MDT_ERR_ARG, "bad flag");
    if (precision < MDT_PREC_FP64 || precision > MDT_PREC_BF16X3) return fail(c, MDT_ERR_ARG, "bad precision");
    if (tc_mode(precision) && c->pes_kind == MDT_PES_EMT) return fail(c, MDT_ERR_UNSUPPORTED, kBf16Scope);
    if ((rc = check_params(c, p, false))) return rc;
    if (c->pes_kind != MDT_PES_EMT) {
        if ((rc = check_nn_ready(c))) return rc;
        if (c->pes_kind == MDT_PES_SURROGATE && (rc = ensure_scratch(c, MDT_PREC_FP64))) return rc;
        const PropParams P = to_dev(c, p);
        const bool surr = c->pes_kind == MDT_PES_SURROGATE;
        if (use_radial(c, precision, false))
            return run_radial(c, P, 0, flag == MDT_ENERGY_ONLY ? 1 : 0, surr, tc_mode(precision));
        if (tc_mode(precision)) return run_tc_generic(c, P, flag == MDT_ENERGY_ONLY ? 1 : 0, tc_mode(precision));
        const bool fast = use_fast(c, precision);
        const LaunchCfg fcfg = fast ? nnf_cfg(c) : LaunchCfg{};
        if (fast && (rc = ensure_mscr(c, fcfg.grid, 0))) return rc;
        cudaError_t e = fast
                            ? launch_nnf(fcfg, c->B, c->M, c->F, c->E, c->X, P, 0,
                                         flag == MDT_ENERGY_ONLY ? 1 : 0, surr)
                            : launch_nn(nn_cfg(c, precision), c->B, c->M, c->E, c->X, P, c->ngeta_max, 0,
                                        flag == MDT_ENERGY_ONLY ? 1 : 0, precision, surr);
        c->launches++;
        return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_calc_force (network)");
    }
    if ((rc = ensure_scratch(c, precision))) return rc;
    const PropParams P = to_dev(c, p);
    cudaError_t e = launch_phase(cfg(c, precision), c->B, c->E, P,
                                 flag == MDT_ENERGY_ONLY ? kPhaseEnergyOnly : kPhaseForce, precision);
    c->launches++;
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_calc_force");
}

int32_t mdt_propagate_1(mdt_ctx *c, const mdt_prop_params *p) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if ((rc = check_params(c, p))) return rc;
    const PropParams P = to_dev(c, p);
    cudaError_t e = launch_phase(cfg(c, 0), c->B, c->E, P, kPhaseProp1, 0);
    c->launches++;
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_propagate_1");
}

int32_t mdt_propagate_2(mdt_ctx *c, const mdt_prop_params *p) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if ((rc = check_params(c, p))) return rc;
    const PropParams P = to_dev(c, p);
    cudaError_t e = launch_phase(cfg(c, 0), c->B, c->E, P, kPhaseProp2, 0);
    c->launches++;
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_propagate_2");
}

int32_t mdt_md_steps(mdt_ctx *c, int32_t nsteps, int32_t precision, const mdt_prop_params *p) {
    int rc = check_ready(c, c && c->pes_kind == MDT_PES_EMT);
    if (rc) return rc;
    if (nsteps < 0) return fail(c, MDT_ERR_ARG, "nsteps < 0");
    if (precision < MDT_PREC_FP64 || precision > MDT_PREC_BF16X3) return fail(c, MDT_ERR_ARG, "bad precision");
    if (tc_mode(precision) && c->pes_kind == MDT_PES_EMT) return fail(c, MDT_ERR_UNSUPPORTED, kBf16Scope);
    if ((rc = check_params(c, p))) return rc;
    if (p->rng_mode == 1 && nsteps > 1) return fail(c, MDT_ERR_ARG, "rng_mode 1 supports one step per call");
    if (c->pes_kind != MDT_PES_EMT) {
        if ((rc = check_nn_ready(c))) return rc;
        if (c->pes_kind == MDT_PES_SURROGATE && (rc = ensure_scratch(c, MDT_PREC_FP64))) return rc;
        if (nsteps == 0) return MDT_OK;
        const PropParams P = to_dev(c, p);
        const bool surr = c->pes_kind == MDT_PES_SURROGATE;
        if (use_radial(c, precision, true)) return run_radial(c, P, nsteps, 2, surr, tc_mode(precision));
        if (tc_mode(precision)) return fail(c, MDT_ERR_UNSUPPORTED, kBf16Scope);
        const bool fast = use_fast(c, precision);
        const LaunchCfg fcfg = fast ? nnf_cfg(c) : LaunchCfg{};
        if (fast && (rc = ensure_mscr(c, fcfg.grid, 0))) return rc;
        cudaError_t e = fast
                            ? launch_nnf(fcfg, c->B, c->M, c->F, c->E, c->X, P, nsteps, 2, surr)
                            : launch_nn(nn_cfg(c, precision), c->B, c->M, c->E, c->X, P, c->ngeta_max, nsteps, 2,
                                        precision, surr);
        c->launches++;
        return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_md_steps (network)");
    }
    if ((rc = ensure_scratch(c, precision))) return rc;
    if (nsteps == 0) return MDT_OK;
    const PropParams P = to_dev(c, p);
    cudaError_t e = launch_md_steps(cfg(c, precision), c->B, c->E, P, nsteps, precision);
    c->launches++;
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_md_steps");
}

int32_t mdt_set_step_limit(mdt_ctx *c, int32_t max_steps) {
    if (!c) return MDT_ERR_ARG;
    if (max_steps < 0) return fail(c, MDT_ERR_ARG, "max_steps < 0");
    c->step_limit = max_steps;
    return MDT_OK;
}

int32_t mdt_refill(mdt_ctx *c, const mdt_refill_params *p, int32_t *generation, int32_t *nrefilled) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!p) return fail(c, MDT_ERR_ARG, "null mdt_refill_params");
    if (!c->have_tmpl) return fail(c, MDT_ERR_STATE, "mdt_refill needs a state uploaded with r and v");
    if (!(p->einc_min > 0.0) || !(p->einc_max >= p->einc_min) || !(p->polar_max >= p->polar_min) ||
        !(p->polar_min >= 0.0) || !(p->polar_max < 90.0) || !std::isfinite(p->z0))
        return fail(c, MDT_ERR_ARG, "mdt_refill: need 0 < einc_min <= einc_max, 0 <= polar_min <= polar_max < 90");
    cudaError_t e = cudaMemsetAsync(c->refill_count, 0, sizeof(int), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->draws, 0xFF, sizeof(double) * 5 * (size_t)c->T, c->stream);  // NaN
    if (e == cudaSuccess)
        e = launch_refill(c->stream, c->B, c->tmpl, c->total_ba, p->z0, p->einc_min, p->einc_max, p->polar_min,
                          p->polar_max, p->azimuth, p->seed, c->gen, c->skok, c->refill_count, c->draws);
    c->launches++;
    int n = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&n, c->refill_count, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && generation)
        e = cudaMemcpyAsync(generation, c->gen, sizeof(int) * c->T, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_refill");
    if (nrefilled) *nrefilled = n;
    if (n > 0 && !c->rfull) c->rnpack = 0;  // restarted trajectories must be in the next pack plan
    return MDT_OK;
}

int32_t mdt_refill_draws(mdt_ctx *c, double *draws) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!draws) return fail(c, MDT_ERR_ARG, "mdt_refill_draws: null output");
    if (!c->draws) return fail(c, MDT_ERR_STATE, "mdt_refill_draws: no refill yet");
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpy(draws, c->draws, sizeof(double) * 5 * (size_t)c->T, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_refill_draws");
}

int32_t mdt_nn_repack(mdt_ctx *c, int32_t *npacks) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!c->R.ok || !c->have_nn) {
        if (npacks) *npacks = 0;
        return MDT_OK;
    }
    std::vector<int> st(c->T);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemcpy(st.data(), c->B.status, sizeof(int) * c->T, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_nn_repack");
    std::vector<int> ids;
    for (int t = 0; t < c->T; ++t)
        if (st[t] == MDT_TRAJ_RUNNING) ids.push_back(t);
    if (!ids.empty() && (int)ids.size() < c->T && !radial_plan(c, ids))
        return fail(c, MDT_ERR_UNSUPPORTED, "mdt_nn_repack: the running trajectories cannot be packed");
    if (npacks) *npacks = c->rnpack;
    return MDT_OK;
}

int32_t mdt_traj_observables(mdt_ctx *c, int32_t *turn_pnts, double *cl_appr, int32_t *cl_appr_step,
                             double *r_min_p) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    const Batch &B = c->B;
    const size_t T = (size_t)c->T;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && turn_pnts) e = cudaMemcpy(turn_pnts, B.obs_turn, sizeof(int) * T, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && cl_appr) e = cudaMemcpy(cl_appr, B.obs_cl, sizeof(double) * T, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && cl_appr_step)
        e = cudaMemcpy(cl_appr_step, B.obs_clstep, sizeof(int) * T, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && r_min_p) e = cudaMemcpy(r_min_p, B.obs_low, sizeof(double) * 3 * T, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_traj_observables");
}

int32_t mdt_set_adsorption(mdt_ctx *c, double start, double end) {
    if (!c) return MDT_ERR_ARG;
    if (!(start <= end)) return fail(c, MDT_ERR_ARG, "mdt_set_adsorption: start must not exceed end");
    c->ads_start = start;
    c->ads_end = end;
    return MDT_OK;
}

int32_t mdt_traj_bounces(mdt_ctx *c, int32_t *bounces, double *interaction_time, int32_t *is_adsorbed,
                         const mdt_prop_params *p) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!p) return fail(c, MDT_ERR_ARG, "mdt_traj_bounces: null parameters");
    const size_t T = (size_t)c->T;
    std::vector<int> h(kObsInts * T);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), c->B.obs_bnc, sizeof(int) * h.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_traj_bounces");
    for (size_t t = 0; t < T; ++t) {
        const int *b = h.data() + kObsInts * t;
        // finalize_bounces as output_scatter calls it before writing (output_mod.f90:660)
        if (bounces) bounces[t] = b[kObsBounces] + std::min(b[kObsPtm], std::min(b[kObsRF], b[kObsVF]));
        if (interaction_time) interaction_time[t] = b[kObsInter] * p->step;
        if (is_adsorbed) is_adsorbed[t] = b[kObsAds];
    }
    return MDT_OK;
}

int32_t mdt_query(mdt_ctx *c, const mdt_prop_params *p, mdt_traj_summary *out) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!out || !p) return fail(c, MDT_ERR_ARG, "mdt_query: null argument");
    const PropParams P = to_dev(c, p);
    cudaError_t e = launch_summary(c->stream, c->B, P, c->summary);
    c->launches++;
    std::vector<double> s(5 * (size_t)c->T);
    std::vector<int> st(c->T);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s.data(), c->summary, sizeof(double) * s.size(), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(st.data(), c->B.status, sizeof(int) * c->T, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_query");
    for (int t = 0; t < c->T; ++t) {
        out[t].status = st[t];
        out[t].steps_done = (int32_t)s[5 * t + 4];
        out[t].epot = s[5 * t + 0];
        out[t].ekin_p = s[5 * t + 1];
        out[t].ekin_l = s[5 * t + 2];
        out[t].ebead = s[5 * t + 3];
    }
    return MDT_OK;
}

int32_t mdt_device_state(mdt_ctx *c, void **ptrs, int64_t *nslots) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!ptrs) return fail(c, MDT_ERR_ARG, "null ptrs");
    Batch &B = c->B;
    void *p[12] = {B.rx, B.ry, B.rz, B.vx, B.vy, B.vz, B.fx, B.fy, B.fz, B.ax, B.ay, B.az};
    for (int k = 0; k < 12; ++k) ptrs[k] = p[k];
    if (nslots) *nslots = c->total_ba;
    return MDT_OK;
}


int32_t mdt_nn_set_model(mdt_ctx *c, const mdt_nn_model *m, int32_t ntypes, const int32_t *z_of_type,
                         int32_t max_neighbors) {
    if (!c) return MDT_ERR_ARG;
    if (!m || !z_of_type || ntypes < 1 || ntypes > kMaxTypes) return fail(c, MDT_ERR_ARG, "mdt_nn_set_model: bad arguments");
    if (m->nelem < 1 || m->nelem > kMaxElem || m->maxsf < 1 || m->maxsf > kMaxSF || m->nlayers < 1 ||
        m->nlayers > kMaxLayers || m->maxnodes < 1 || m->maxnodes > kMaxNodes)
        return fail(c, MDT_ERR_UNSUPPORTED, "network larger than 4 elements / 64 functions / 4 layers of 64 nodes");
    NNDev M{};
    M.nelem = m->nelem;
    M.maxsf = m->maxsf;
    M.nlayers = m->nlayers;
    M.maxnodes = kMaxNodes;
    M.maxweights = m->maxweights;
    M.maxnb = max_neighbors > 0 ? max_neighbors : 192;
    M.cutoff_type = m->cutoff_type;
    M.cutoff_alpha = m->cutoff_alpha;
    M.scalesym = m->scalesym;
    M.centersym = m->centersym;
    M.normnodes = m->normnodes;
    M.remove_atom_energies = m->remove_atom_energies;
    M.scmin = m->scmin;
    M.scmax = m->scmax;
    M.margin = (float)c->margin;
    if (M.cutoff_type < 0 || M.cutoff_type > 8) return fail(c, MDT_ERR_ARG, "cutoff_type must be 0..8");
    for (int t = 0; t < kMaxTypes; ++t) M.elem_of_type[t] = -1;
    for (int t = 0; t < ntypes; ++t)
        for (int e = 0; e < m->nelem; ++e)
            if (z_of_type[t] != 0 && m->z[e] == z_of_type[t]) M.elem_of_type[t] = e;
    const int ne = m->nelem, ms = m->maxsf;
    std::vector<int> e1(ne * ms, -1), e2(ne * ms, -1), izeta(ne * ms, -1), etaslot(ne * ms, 0);
    std::vector<double> pnorm(ne * ms, 1.0);
    auto elem_of_z = [&](int z) {
        for (int e = 0; e < ne; ++e)
            if (m->z[e] == z) return e;
        return -1;
    };
    int ngmax = 0;
    M.maxcut = 0.0;
    for (int e = 0; e < ne; ++e) {
        const int nsf = m->nsf[e];
        if (nsf < 1 || nsf > ms) return fail(c, MDT_ERR_ARG, "bad symmetry-function count");
        M.nsf[e] = nsf;
        M.rc[e] = m->rc[e * ms];
        int ng = 0, ng3 = 0;
        for (int s = 0; s < nsf; ++s) {
            const int k = e * ms + s;
            if (m->sftype[k] != 2 && m->sftype[k] != 3)
                return fail(c, MDT_ERR_UNSUPPORTED, "only symmetry-function types 2 and 3 are supported");
            if (m->rc[k] != M.rc[e])
                return fail(c, MDT_ERR_UNSUPPORTED, "all symmetry functions of an element must share one cutoff");
            e1[k] = elem_of_z(m->e1[k]);
            if (m->sftype[k] == 3) {
                ++ng3;
                e2[k] = elem_of_z(m->e2[k]);
                const double zm1 = m->zeta[k] - 1.0;
                if (zm1 >= 0.0 && zm1 <= 64.0 && zm1 == std::floor(zm1)) izeta[k] = (int)zm1;
                pnorm[k] = std::pow(2.0, 1.0 - m->zeta[k]);
                int slot = -1;
                for (int q = 0; q < ng; ++q)
                    if (M.g3eta[e][q] == m->eta[k]) slot = q;
                if (slot < 0) {
                    if (ng >= kMaxEta) return fail(c, MDT_ERR_UNSUPPORTED, "more than 6 distinct G3 eta values");
                    M.g3eta[e][ng] = m->eta[k];
                    slot = ng++;
                }
                etaslot[k] = slot;
            }
        }
        if (ng3 > 24) return fail(c, MDT_ERR_UNSUPPORTED, "more than 24 G3 functions per element");
        M.ng3eta[e] = ng;
        ngmax = std::max(ngmax, ng);
        M.maxcut = std::max(M.maxcut, M.rc[e]);
        int off = 0;
        for (int l = 0; l <= m->nlayers; ++l) {
            M.nodes[e][l] = m->nodes[e * (m->nlayers + 1) + l];
            if (M.nodes[e][l] < 1 || M.nodes[e][l] > kMaxNodes) return fail(c, MDT_ERR_ARG, "bad node count");
        }
        if (M.nodes[e][0] != nsf || M.nodes[e][m->nlayers] != 1) return fail(c, MDT_ERR_ARG, "bad layer sizes");
        for (int l = 1; l <= m->nlayers; ++l) {
            M.woff[e][l] = off;
            off += M.nodes[e][l - 1] * M.nodes[e][l] + M.nodes[e][l];
        }
        if (off > m->maxweights) return fail(c, MDT_ERR_ARG, "maxweights smaller than the network");
        M.atom_energy[e] = (m->remove_atom_energies && m->atom_energy) ? m->atom_energy[e] : 0.0;
    }
    // grid form of the G3 functions (see NNDev::g3fast)
    for (int e = 0; e < ne; ++e) {
        M.g3fast[e] = 0;
        M.nlz[e] = 0;
        for (int g = 0; g < 4; ++g)
            for (int q = 0; q < 8; ++q) M.sf_of[e][g][q] = -1;
        bool ok = M.ng3eta[e] <= 4;
        int pe1 = -2, pe2 = -2, nq = 0;
        for (int s = 0; s < M.nsf[e] && ok; ++s) {
            const int k = e * ms + s;
            if (m->sftype[k] != 3) continue;
            if (izeta[k] < 0 || izeta[k] > 31) { ok = false; break; }
            if (pe1 == -2) { pe1 = e1[k]; pe2 = e2[k]; }
            if (!((e1[k] == pe1 && e2[k] == pe2) || (e1[k] == pe2 && e2[k] == pe1))) { ok = false; break; }
            int q = -1;
            for (int r = 0; r < nq; ++r)
                if (M.lz_lam[e][r] == (float)m->lambda[k] && M.lz_zm1[e][r] == izeta[k]) q = r;
            if (q < 0) {
                if (nq >= 8) { ok = false; break; }
                q = nq++;
                M.lz_lam[e][q] = (float)m->lambda[k];
                M.lz_zm1[e][q] = izeta[k];
                M.lz_zl[e][q] = (float)(m->zeta[k] * m->lambda[k]);
                M.lz_pnorm[e][q] = (float)pnorm[k];
            }
            if (M.sf_of[e][etaslot[k]][q] != -1) { ok = false; break; }
            M.sf_of[e][etaslot[k]][q] = (int8_t)s;
        }
        if (ok && pe1 != -2) {
            M.g3fast[e] = 1;
            M.nlz[e] = nq;
            M.g3pair[e][0] = pe1;
            M.g3pair[e][1] = pe2;
        }
    }
    std::vector<uint8_t> act((size_t)ne * kMaxLayers * kMaxNodes, 'l');
    for (int e = 0; e < ne; ++e)
        for (int l = 0; l < m->nlayers; ++l)
            for (int n = 0; n < M.nodes[e][l + 1]; ++n) {
                const uint8_t a = m->act[((size_t)e * m->nlayers + l) * m->maxnodes + n];
                if (!std::strchr("tglcsSeph", (int)a) || a == 0) return fail(c, MDT_ERR_ARG, "unknown activation");
                act[((size_t)e * kMaxLayers + l) * kMaxNodes + n] = a;
            }
    std::vector<float> wf((size_t)ne * m->maxweights);
    for (size_t k = 0; k < wf.size(); ++k) wf[k] = (float)m->weights[k];
    // device copies
    for (void *p : c->nnbufs) cudaFree(p);
    c->nnbufs.clear();
    cudaError_t e = cudaSuccess;
    auto up = [&](const void *src, size_t bytes) -> void * {
        void *d = nullptr;
        if (e != cudaSuccess) return nullptr;
        e = cudaMalloc(&d, std::max<size_t>(bytes, 16));
        if (e != cudaSuccess) return nullptr;
        c->nnbufs.push_back(d);
        e = cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice);
        return d;
    };
    const size_t nk = (size_t)ne * ms;
    M.sftype = (const int *)up(m->sftype, 4 * nk);
    M.e1 = (const int *)up(e1.data(), 4 * nk);
    M.e2 = (const int *)up(e2.data(), 4 * nk);
    M.izeta = (const int *)up(izeta.data(), 4 * nk);
    M.etaslot = (const int *)up(etaslot.data(), 4 * nk);
    M.eta = (const double *)up(m->eta, 8 * nk);
    M.rs = (const double *)up(m->rshift, 8 * nk);
    M.lam = (const double *)up(m->lambda, 8 * nk);
    M.zeta = (const double *)up(m->zeta, 8 * nk);
    M.pnorm = (const double *)up(pnorm.data(), 8 * nk);
    M.smin = (const double *)up(m->smin, 8 * nk);
    M.smax = (const double *)up(m->smax, 8 * nk);
    M.savg = (const double *)up(m->savg, 8 * nk);
    M.act = (const uint8_t *)up(act.data(), act.size());
    M.wd = (const double *)up(m->weights, 8 * (size_t)ne * m->maxweights);
    M.wf = (const float *)up(wf.data(), 4 * wf.size());
    std::vector<float4> g2tab;
    FastNN F = build_fast(M, m, e1, etaslot, g2tab);
    if (F.ok) {
        std::vector<float> zeros(5 * nk, 0.f);
        F.scal = (const float4 *)up(zeros.data(), 16 * nk);
        F.dscal = (const float *)up(zeros.data(), 4 * nk);
        F.g2tab = (const float4 *)up(g2tab.data(), sizeof(float4) * g2tab.size());
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_nn_set_model upload");
    c->F = F;
    c->R = build_radial(M, m, F, e1);
    c->R.wf = M.wf;
    c->R.fscal = F.scal;
    c->R.fdscal = F.dscal;
    c->RG = build_tc_generic(M, m, F);
    c->RG.wf = M.wf;
    c->RG.fscal = F.scal;
    c->RG.fdscal = F.dscal;
    c->rnpack = c->rblock = 0;
    c->d_scal = (float4 *)F.scal;
    c->d_dscal = (float *)F.dscal;
    c->h_smin.assign(m->smin, m->smin + nk);
    c->h_smax.assign(m->smax, m->smax + nk);
    c->h_savg.assign(m->savg, m->savg + nk);
    c->M = M;
    c->ngeta_max = ngmax;
    c->have_nn = true;
    c->X = NNScratch{};  // re-allocated for the new neighbour bound on next use
    c->nn_maxnb_alloc = 0;
    c->skin_dirty = true;
    return upload_fast_scaling(c);
}

int32_t mdt_set_pes(mdt_ctx *c, int32_t pes_kind, double range_margin) {
    if (!c) return MDT_ERR_ARG;
    if (pes_kind != MDT_PES_EMT && pes_kind != MDT_PES_NENE && pes_kind != MDT_PES_SURROGATE)
        return fail(c, MDT_ERR_ARG, "unknown PES kind");
    if (!(range_margin >= 0.0)) return fail(c, MDT_ERR_ARG, "range margin must be >= 0");
    c->pes_kind = pes_kind;
    c->margin = range_margin;
    c->M.margin = (float)range_margin;
    return c->have_nn ? upload_fast_scaling(c) : MDT_OK;
}

int32_t mdt_nn_set_skin(mdt_ctx *c, double skin_ang) {
    if (!c) return MDT_ERR_ARG;
    if (!(skin_ang >= 0.0) || skin_ang > 5.0) return fail(c, MDT_ERR_ARG, "skin must be in [0, 5] A");
    c->skin_ang = skin_ang;
    c->skin_dirty = true;
    c->rnpack = 0;  // the thread-per-atom plan checks cell widths against the skin cutoff
    return MDT_OK;
}

int32_t mdt_nn_radial_kernel(mdt_ctx *c, int32_t enable) {
    if (!c) return MDT_ERR_ARG;
    c->radial_enabled = enable != 0;
    return c->have_nn && c->R.ok ? 1 : 0;
}

int32_t mdt_nn_radial_block(mdt_ctx *c, int32_t max_block) {
    if (!c) return MDT_ERR_ARG;
    if (max_block < 32 || max_block > kRBlockMax) return fail(c, MDT_ERR_ARG, "max_block outside [32, 512]");
    c->rmaxblock = max_block;
    c->rnpack = 0;  // re-plan on the next evaluation
    return MDT_OK;
}

// Autotuner of the thread-per-atom kernel: times `nsteps` fused MD steps of the current
// batch for every candidate (largest CTA in {256, 384, 512} atoms -- the pack plan's block
// cap, which sets the waves and the warps per SM -- times Verlet skin in {0.3, 0.5, 0.75, 1.0}
// A), each from the same saved state, keeps the fastest and puts the state back.
int32_t mdt_autotune(mdt_ctx *c, int32_t precision, int32_t nsteps, const mdt_prop_params *p, int32_t *block,
                     double *skin_ang, double *ms_per_step) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!p || nsteps < 1) return fail(c, MDT_ERR_ARG, "mdt_autotune: parameters and nsteps >= 1 needed");
    if (c->pes_kind == MDT_PES_EMT) return fail(c, MDT_ERR_UNSUPPORTED, "mdt_autotune tunes the network kernels");
    if ((rc = check_nn_ready(c))) return rc;
    if (!use_radial(c, precision, true))
        return fail(c, MDT_ERR_UNSUPPORTED, "mdt_autotune: the batch does not run on the thread-per-atom kernel");
    // saved state: r, v, a, f, dens (per bead-atom), epot (per bead), status, steps, observables
    Batch &B = c->B;
    const size_t nba = (size_t)c->total_ba, T = (size_t)c->T, nbd = (size_t)c->total_beads;
    double *d12[13] = {B.rx, B.ry, B.rz, B.vx, B.vy, B.vz, B.ax, B.ay, B.az, B.fx, B.fy, B.fz, B.dens};
    int *ivec[2] = {B.status, B.steps_done};
    const size_t obs_i = (3 + kObsInts) * T, obs_d = (4 + kObsDots) * T;
    const size_t bytes = 8 * (13 * nba + nbd + obs_d) + 4 * (2 * T + obs_i + 2 * T);
    unsigned char *snap = nullptr;
    cudaError_t e = cudaMalloc(&snap, bytes);
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_autotune snapshot");
    auto copy_all = [&](bool save) -> cudaError_t {
        size_t off = 0;
        cudaError_t err = cudaSuccess;
        auto mv = [&](void *dev, size_t n) {
            if (err == cudaSuccess)
                err = cudaMemcpyAsync(save ? snap + off : dev, save ? dev : snap + off, n, cudaMemcpyDeviceToDevice,
                                      c->stream);
            off += n;
        };
        for (double *a : d12) mv(a, 8 * nba);
        mv(B.epot, 8 * nbd);
        mv(B.obs_cl, 8 * obs_d);  // obs_cl, obs_low, obs_dot are one allocation
        for (int *a : ivec) mv(a, 4 * T);
        mv(B.obs_turn, 4 * obs_i);  // obs_turn, obs_up, obs_clstep, obs_bnc likewise
        mv(c->X.fallback, 4 * T);
        mv(c->X.nnstatus, 4 * T);
        return err;
    };
    e = copy_all(true);
    const int keep_block = c->rmaxblock;
    const double keep_skin = c->skin_ang;
    const PropParams P = to_dev(c, p);
    const bool surr = c->pes_kind == MDT_PES_SURROGATE;
    const int tc = tc_mode(precision);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int blocks[3] = {256, 384, 512};
    const double skins[4] = {0.3, 0.5, 0.75, 1.0};
    double best = 1e300;
    int bb = keep_block;
    double bs = keep_skin;
    for (int ib = 0; ib < 3 && e == cudaSuccess; ++ib) {
        if (blocks[ib] < ((c->max_atoms + 31) & ~31)) continue;
        for (int is = 0; is < 4 && e == cudaSuccess; ++is) {
            c->rmaxblock = blocks[ib];
            c->skin_ang = skins[is];
            c->skin_dirty = true;
            c->rnpack = 0;
            if (!use_radial(c, precision, true)) continue;
            e = copy_all(false);
            if (e != cudaSuccess) break;
            if ((rc = run_radial(c, P, 2, 2, surr, tc))) break;  // warm-up: lists built, code loaded
            e = cudaEventRecord(e0, c->stream);
            if (e == cudaSuccess && (rc = run_radial(c, P, nsteps, 2, surr, tc))) break;
            if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e == cudaSuccess && ms < best) {
                best = ms;
                bb = blocks[ib];
                bs = skins[is];
            }
        }
    }
    c->rmaxblock = best < 1e300 ? bb : keep_block;
    c->skin_ang = best < 1e300 ? bs : keep_skin;
    c->skin_dirty = true;
    c->rnpack = 0;
    if (e == cudaSuccess) e = copy_all(false);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(snap);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_autotune");
    if (best >= 1e300) return fail(c, MDT_ERR_UNSUPPORTED, "mdt_autotune: no candidate ran");
    if (block) *block = c->rmaxblock;
    if (skin_ang) *skin_ang = c->skin_ang;
    if (ms_per_step) *ms_per_step = best / nsteps;
    return MDT_OK;
}

int32_t mdt_nn_fast_path(mdt_ctx *c, int32_t enable) {
    if (!c) return MDT_ERR_ARG;
    c->fast_enabled = enable != 0;
    return c->have_nn && c->F.ok ? 1 : 0;
}

int32_t mdt_nn_stats(mdt_ctx *c, int32_t *fallbacks, int32_t *overflow) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!c->X.nbw) return fail(c, MDT_ERR_STATE, "no network evaluation yet");
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (fallbacks && e == cudaSuccess)
        e = cudaMemcpy(fallbacks, c->X.fallback, sizeof(int) * c->T, cudaMemcpyDeviceToHost);
    if (overflow && e == cudaSuccess) e = cudaMemcpy(overflow, c->X.nnstatus, sizeof(int) * c->T, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_nn_stats");
}

int32_t mdt_nn_neighbors(mdt_ctx *c, int32_t *counts, int32_t *words) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!c->X.nbw) return fail(c, MDT_ERR_STATE, "no network evaluation yet");
    cudaError_t e = cudaStreamSynchronize(c->stream);
    int a = 0;
    for (int t = 0; t < c->T && e == cudaSuccess; ++t) {
        const int N = c->natoms[t];
        const int64_t base = c->ba_off[t];  // bead 0
        if (counts) e = cudaMemcpy(counts + a, c->X.nbcnt + base, sizeof(int) * N, cudaMemcpyDeviceToHost);
        if (words && e == cudaSuccess)
            e = cudaMemcpy(words + (size_t)a * c->M.maxnb, c->X.nbw + base * c->M.maxnb,
                           sizeof(int) * (size_t)N * c->M.maxnb, cudaMemcpyDeviceToHost);
        a += N;
    }
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_nn_neighbors");
}


int32_t mdt_nn_descriptors(mdt_ctx *c, int32_t precision, double *G) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!G) return fail(c, MDT_ERR_ARG, "null output");
    if ((rc = check_nn_ready(c))) return rc;
    cudaError_t e = cudaSuccess;
    double *d = dalloc<double>(c, (size_t)c->total_ba * c->M.maxsf, e);
    if (!d) return fail(c, MDT_ERR_NOMEM, "descriptor buffer");
    e = cudaMemsetAsync(d, 0, sizeof(double) * c->total_ba * c->M.maxsf, c->stream);
    NNScratch X = c->X;
    X.gout = d;
    mdt_prop_params p{};
    p.step = 1.0;
    const PropParams P = to_dev(c, &p);
    if (e == cudaSuccess)
        e = launch_nn(nn_cfg(c, precision), c->B, c->M, c->E, X, P, c->ngeta_max, 0, 1, precision, false);
    c->launches++;
    std::vector<double> h((size_t)c->total_ba * c->M.maxsf);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_nn_descriptors");
    // device slot order (bead-major) -> Fortran (nb, N) order per trajectory
    const int ms = c->M.maxsf;
    for (int t = 0; t < c->T; ++t) {
        const int N = c->natoms[t], nb = c->nbeads[t];
        for (int b = 0; b < nb; ++b)
            for (int i = 0; i < N; ++i) {
                const int64_t src = c->ba_off[t] + (int64_t)b * N + i, dst = c->ba_off[t] + (int64_t)i * nb + b;
                std::memcpy(G + dst * ms, h.data() + src * ms, sizeof(double) * ms);
            }
    }
    return MDT_OK;
}


int32_t mdt_train_set_labels(mdt_ctx *c, const double *energy, const double *forces) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!energy || !forces) return fail(c, MDT_ERR_ARG, "null labels");
    if (!c->have_nn) return fail(c, MDT_ERR_STATE, "no network installed (call mdt_nn_set_model)");
    if (c->max_beads != 1) return fail(c, MDT_ERR_ARG, "training configurations must have one bead");
    if (!c->M.scalesym || c->M.centersym || c->M.normnodes)
        return fail(c, MDT_ERR_UNSUPPORTED, "training needs scale_symmetry_functions without centering/normalize_nodes");
    if ((rc = ensure_nn_scratch(c))) return rc;
    cudaError_t e = cudaSuccess;
    const size_t nw = (size_t)c->M.nelem * c->M.maxweights;
    c->t_E = dalloc<double>(c, c->T, e);
    c->t_fx = dalloc<double>(c, c->total_ba, e);
    c->t_fy = dalloc<double>(c, c->total_ba, e);
    c->t_fz = dalloc<double>(c, c->total_ba, e);
    c->t_G = dalloc<double>(c, (size_t)c->total_ba * c->M.maxsf, e);
    c->t_grad = dalloc<double>(c, nw, e);
    c->t_loss = dalloc<double>(c, 4, e);
    c->t_theta = dalloc<float>(c, nw, e);
    c->t_m = dalloc<float>(c, nw, e);
    c->t_v = dalloc<float>(c, nw, e);
    c->t_conf = dalloc<int>(c, c->T, e);
    if (!c->t_E || !c->t_fx || !c->t_fy || !c->t_fz || !c->t_G || !c->t_grad || !c->t_loss || !c->t_theta ||
        !c->t_m || !c->t_v || !c->t_conf)
        return fail(c, MDT_ERR_NOMEM, "training buffers");
    e = cudaMemcpyAsync(c->t_E, energy, sizeof(double) * c->T, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->stage, forces, sizeof(double) * 3 * c->total_ba, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = launch_unpack(c->stream, c->B, c->stage, c->t_fx, c->t_fy, c->t_fz, c->total_ba, c->ba_traj);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->t_G, 0, sizeof(double) * c->total_ba * c->M.maxsf, c->stream);
    // raw symmetry functions and neighbour lists, computed once
    NNScratch X = c->X;
    X.gout = c->t_G;
    mdt_prop_params p{};
    p.step = 1.0;
    const PropParams P = to_dev(c, &p);
    if (e == cudaSuccess) e = launch_nn(nn_cfg(c, MDT_PREC_FP64), c->B, c->M, c->E, X, P, c->ngeta_max, 0, 1,
                                        MDT_PREC_FP64, false);
    c->launches += 2;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->t_theta, c->M.wf, sizeof(float) * nw, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->t_m, 0, sizeof(float) * nw, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->t_v, 0, sizeof(float) * nw, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "mdt_train_set_labels");
    c->t_step = 0;
    c->have_labels = true;
    return MDT_OK;
}

static int train_run(mdt_ctx *c, const mdt_train_opts *o, const int32_t *conf, int32_t n, bool update,
                     double *stats, double *grad_out) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!c->have_labels) return fail(c, MDT_ERR_STATE, "no training labels (call mdt_train_set_labels)");
    if (!o || !conf || n < 1 || n > c->T) return fail(c, MDT_ERR_ARG, "bad training arguments");
    if (o->precision < MDT_PREC_FP64 || o->precision > MDT_PREC_BF16X3) return fail(c, MDT_ERR_ARG, "bad precision");
    const bool gemm = o->precision == MDT_PREC_BF16 || o->precision == MDT_PREC_BF16X3;
    if (gemm) {
        if (c->M.nlayers != 3 || c->M.nelem > 2)
            return fail(c, MDT_ERR_UNSUPPORTED, "BF16 GEMM training: networks of two hidden layers, at most two elements");
        for (int e = 0; e < c->M.nelem; ++e)
            if (c->M.nodes[e][0] > 48 || c->M.nodes[e][1] > 32 || c->M.nodes[e][2] > 32 || c->M.nodes[e][3] != 1)
                return fail(c, MDT_ERR_UNSUPPORTED, "BF16 GEMM training: <= 48 descriptors, <= 32 nodes per hidden layer");
    }
    for (int k = 0; k < n; ++k)
        if (conf[k] < 0 || conf[k] >= c->T) return fail(c, MDT_ERR_ARG, "configuration index out of range");
    const size_t nw = (size_t)c->M.nelem * c->M.maxweights;
    cudaError_t e = cudaMemcpyAsync(c->t_conf, conf, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->t_grad, 0, sizeof(double) * nw, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->t_loss, 0, sizeof(double) * 4, c->stream);
    TrainArgs A{c->t_E, c->t_fx, c->t_fy, c->t_fz, c->t_G, c->t_conf, n, o->w_energy, o->w_force, c->t_theta,
                c->t_grad, c->t_loss};
    GemmTrain G{};
    if (gemm && e == cudaSuccess) {
        // rows: the atoms of the step's configurations, element 0 first
        std::vector<int> rows[2];
        for (int k = 0; k < n; ++k) {
            const int t = conf[k];
            for (int i = 0; i < c->natoms[t]; ++i) {
                const int el = c->M.elem_of_type[c->h_type[c->atom_off[t] + i]];
                if (el >= 0) rows[el].push_back((int)(c->ba_off[t] + i));
            }
        }
        std::vector<int> slot(rows[0]);
        slot.insert(slot.end(), rows[1].begin(), rows[1].end());
        const int R = (int)slot.size();
        if (R > c->g_cap) {
            const int cap = std::max(R, 2 * c->g_cap);
            c->g_slot = dalloc<int>(c, (size_t)cap, e);
            c->g_f = dalloc<float>(c, gemm_train_floats(cap), e);
            c->g_b = dalloc<__nv_bfloat16>(c, 2 * gemm_train_bf16(cap), e);  // high and low parts
            if (!c->g_gw) c->g_gw = dalloc<float>(c, gemm_train_gw(cap), e);
            if (!c->g_slot || !c->g_f || !c->g_b || !c->g_gw) return fail(c, MDT_ERR_NOMEM, "GEMM training buffers");
            c->g_cap = cap;
        }
        const size_t nsl = (size_t)c->total_ba * c->M.maxsf;
        if (!c->g_dg) c->g_dg = dalloc<float>(c, nsl, e);
        if (!c->g_xdot) c->g_xdot = dalloc<float>(c, nsl, e);
        if (!c->g_eat) c->g_eat = dalloc<double>(c, (size_t)c->total_ba, e);
        if (!c->g_arow) c->g_arow = dalloc<double>(c, (size_t)c->total_ba, e);
        if (!c->g_dg || !c->g_xdot || !c->g_eat || !c->g_arow) return fail(c, MDT_ERR_NOMEM, "GEMM training buffers");
        if (!c->cublas) {
            if (cublasCreate(&c->cublas) != CUBLAS_STATUS_SUCCESS) return fail(c, MDT_ERR_CUDA, "cublasCreate failed");
        }
        if (R > 0) e = cudaMemcpyAsync(c->g_slot, slot.data(), sizeof(int) * R, cudaMemcpyHostToDevice, c->stream);
        G.slot = c->g_slot;
        G.rows[0] = 0;
        G.rows[1] = (int)rows[0].size();
        G.rows[2] = R;
        G.R = R;
        G.M = c->M;
        G.theta = c->t_theta;
        G.G = c->t_G;
        G.dg = c->g_dg;
        G.eat = c->g_eat;
        G.xdot = c->g_xdot;
        G.arow = c->g_arow;
        G.grad = c->t_grad;
        gemm_train_carve(G, c->g_f, c->g_b, c->g_gw, c->g_cap);
        G.split = o->precision == MDT_PREC_BF16X3 ? 1 : 0;
        if (e == cudaSuccess && R > 0 && gemm_train_forward(c->cublas, c->stream, G))
            return fail(c, MDT_ERR_CUDA, "BF16 GEMM training: forward products failed");
        A.dgin = c->g_dg;
        A.eatin = c->g_eat;
        A.xdot = c->g_xdot;
        A.arow = c->g_arow;
        c->launches += 6;
    }
    if (e == cudaSuccess)
        e = launch_train(c->stream, c->num_sms, c->B, c->M, c->X, A, c->max_atoms, c->ngeta_max, c->counter,
                         gemm ? MDT_PREC_FP32 : o->precision);
    c->launches++;
    if (gemm && e == cudaSuccess && G.R > 0) {
        if (gemm_train_backward(c->cublas, c->stream, G))
            return fail(c, MDT_ERR_CUDA, "BF16 GEMM training: tangent and gradient products failed");
        c->launches += 6;
    }
    if (update && e == cudaSuccess) {
        ++c->t_step;
        e = launch_adam(c->stream, c->t_theta, c->t_m, c->t_v, c->t_grad, (int)nw, 1.0 / n, o->lr, o->beta1, o->beta2,
                        o->eps, c->t_step, nullptr);
        c->launches++;
    }
    double loss[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(loss, c->t_loss, sizeof(loss), cudaMemcpyDeviceToHost, c->stream);
    std::vector<double> g;
    if (grad_out && e == cudaSuccess) {
        g.resize(nw);
        e = cudaMemcpyAsync(g.data(), c->t_grad, sizeof(double) * nw, cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "training step");
    if (stats) {
        stats[0] = loss[3] > 0 ? loss[0] / loss[3] : 0.0;
        stats[1] = loss[2] > 0 ? loss[1] / loss[2] : 0.0;
        stats[2] = o->w_energy * stats[0] + o->w_force * stats[1];
    }
    if (grad_out)
        for (size_t k = 0; k < nw; ++k) grad_out[k] = g[k] / n;
    return MDT_OK;
}

int32_t mdt_train_step(mdt_ctx *c, const mdt_train_opts *opts, const int32_t *conf_ids, int32_t n, double *stats) {
    return train_run(c, opts, conf_ids, n, true, stats, nullptr);
}

int32_t mdt_train_gradient(mdt_ctx *c, const mdt_train_opts *opts, const int32_t *conf_ids, int32_t n,
                           double *grad) {
    if (!grad) return c ? fail(c, MDT_ERR_ARG, "null gradient output") : MDT_ERR_ARG;
    return train_run(c, opts, conf_ids, n, false, nullptr, grad);
}

int32_t mdt_train_commit(mdt_ctx *c, double *weights) {
    int rc = check_ready(c, false);
    if (rc) return rc;
    if (!c->have_labels) return fail(c, MDT_ERR_STATE, "nothing trained");
    const int nw = c->M.nelem * c->M.maxweights;
    cudaError_t e = launch_weights_to_model(c->stream, c->t_theta, const_cast<float *>(c->M.wf),
                                            const_cast<double *>(c->M.wd), nw);
    c->launches++;
    if (weights && e == cudaSuccess)
        e = cudaMemcpyAsync(weights, c->M.wd, sizeof(double) * nw, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? MDT_OK : cuda_fail(c, e, "mdt_train_commit");
}

}  // extern "C"
