// mdt_internal.h -- launchers shared between the engine's translation units.
#pragma once
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mdt_common.cuh"
#include "mdt_nn.cuh"

namespace mdt {

struct LaunchCfg {
    cudaStream_t stream;
    int grid;
    const int *order;  // trajectory work order (largest first)
    int *counter;      // device work-queue counter (reset by the launcher)
};

cudaError_t launch_phase(const LaunchCfg &c, const Batch &B, const EmtConst &E, const PropParams &P, int phase,
                         int precision);
cudaError_t launch_md_steps(const LaunchCfg &c, const Batch &B, const EmtConst &E, const PropParams &P, int nsteps,
                            int precision);
cudaError_t launch_unpack(cudaStream_t s, const Batch &B, const double *src, double *x, double *y, double *z,
                          int64_t total_ba, const int *ba_traj);
cudaError_t launch_unpack_state(cudaStream_t s, const Batch &B, const double *sr, const double *sv, double *tmpl,
                                int64_t total_ba, const int *ba_traj);
cudaError_t launch_pack_state(cudaStream_t s, const Batch &B, double *dr, double *dv, double *df, double *da,
                              int64_t total_ba, const int *ba_traj);
cudaError_t launch_pack_scalar(cudaStream_t s, const Batch &B, double *dst, const double *x, int64_t total_ba,
                               const int *ba_traj);
cudaError_t launch_summary(cudaStream_t s, const Batch &B, const PropParams &P, double *out5);
int max_resident_ctas(int max_atoms, int max_beads, int precision);

cudaError_t launch_nn(const LaunchCfg &c, const Batch &B, const NNDev &M, const EmtConst &E, const NNScratch &X,
                      const PropParams &P, int ngeta, int nsteps, int mode, int precision, bool surrogate);
int nn_resident_ctas(const NNDev &M, int max_atoms, int max_beads, int ngeta, int precision, bool surrogate);

// FP32 fast path (mdt_nnf.cu)
int nnf_zm_supported(int zm);
size_t nnf_total_smem(const Batch &B, const NNDev &M, const FastNN &F);
int nnf_warps_per_cta();
int nnf_resident_ctas(const Batch &B, const NNDev &M, const FastNN &F);
cudaError_t launch_nnf(const LaunchCfg &c, const Batch &B, const NNDev &M, const FastNN &F, const EmtConst &E,
                       const NNScratch &X, const PropParams &P, int nsteps, int mode, bool surrogate);

// derived EMT constants (mdt_noalloc.cu), shared by both EMT entry points
int emt_derive_constants(int32_t ntypes, const double *eta2, const double *n0, const double *e0,
                         const double *lambda, const double *v0, const double *kappa, const double *s0,
                         const int32_t *pes, EmtConst &E);

cudaError_t launch_obs_reset(cudaStream_t s, const Batch &B);
cudaError_t launch_refill(cudaStream_t s, const Batch &B, const double *tmpl, int64_t total_ba, double z0,
                          double emin, double emax, double pmin, double pmax, double azimuth, uint64_t seed,
                          int *gen, int *skok, int *count, double *draws);

// FP32 thread-per-atom kernel of radial-only models (mdt_nnr.cu)
// shape of a model (group counts, hidden layers; maxbl[g] = longest recurrence block group g
// admits, 0 = none): sets R.ka, R.kb, R.bla, R.blb
bool nnr_shape(int cnt0, int cnt1, int nh, const int *maxbl, RadialNN &R);
size_t nnr_smem(const RadialNN &R);
size_t nnr_hb_bytes(const RadialNN &R);  // network buffer / tensor-core operand area (EMT fallback area)
size_t nnr_emt_smem(int max_atoms);  // EMT fallback area (aliases the network buffers)
int nnr_resident_ctas(const RadialNN &R);
// network of a generic model (R from build_tc_generic: nin 24 or 48, nh 1 or 2, R.tc 1 or 2)
// on the tensor cores for every bead-atom: raw descriptors G [ba][maxsf] in, atomic energies
// (Ha) and dE/dG out; one CTA per SM (the CTA holds all of its SM's TMEM)
cudaError_t launch_nn_tc(cudaStream_t s, int grid, const Batch &B, const RadialNN &R, const double *G,
                         const int *ba_traj, int64_t total_ba, float *dg, double *eat, int *err, int do_forces);
size_t nn_tc_smem(int nin, int nh, int tc);
// the constant-friction Langevin coefficients of every single-bead slot (8 per slot) for
// the propagation parameters P: the thread-per-atom kernel reads them instead of forming
// them (FP64 exp, sqrt and divisions) for every pack of every launch
cudaError_t launch_nnr_lcoef(cudaStream_t s, const Batch &B, const PropParams &P, const int *ba_traj,
                             int64_t total_ba, double *lcoef);
cudaError_t launch_nnr(const LaunchCfg &c, const Batch &B, const RadialNN &R, const EmtConst &E, const NNScratch &X,
                       const PropParams &P, const int2 *packs, const int *ptraj, int npack, int nsteps, int mode);

struct TrainArgs {
    const double *E_ref;
    const double *fx_ref, *fy_ref, *fz_ref;
    const double *G;
    const int *conf;
    int nconf;
    double wE, wF;
    const float *theta;
    double *grad;
    double *loss;
    // network outside the kernel (BF16 GEMM training): per slot dE/dG [slot][maxsf] and the
    // output-node value in, the scaled descriptor tangent [slot][maxsf] and dL/dE of the
    // slot's configuration out; the kernel then runs descriptors, forces, loss and tangent only
    const float *dgin = nullptr;
    const double *eatin = nullptr;
    float *xdot = nullptr;
    double *arow = nullptr;
};
cudaError_t launch_train(cudaStream_t s, int num_sms, const Batch &B, const NNDev &M, const NNScratch &X,
                         const TrainArgs &A, int max_atoms, int ngeta, int *counter, int precision);
// The network of a training step as BF16 GEMMs (mdt_train_gemm.cu): rows = the atoms of the
// step's configurations ordered by element (rows[e]..rows[e+1]), slot[r] their bead-atom
// slots; row arrays carved from one FP32 and one BF16 pool (gemm_train_carve)
struct GemmTrain {
    const int *slot = nullptr;
    int rows[3] = {0, 0, 0};
    int R = 0;
    NNDev M{};
    const float *theta = nullptr;  // live FP32 master weights
    const double *G = nullptr;     // raw descriptors [slot][maxsf]
    float *dg = nullptr;           // dE/dG [slot][maxsf] (out)
    double *eat = nullptr;         // output node per slot (out)
    float *xdot = nullptr;         // scaled descriptor tangent [slot][maxsf] (in)
    double *arow = nullptr;        // dL/dE per slot (in)
    double *grad = nullptr;        // gradient (FP64, += )
    struct {
        float *x, *cv, *z1, *h1, *z2, *h2, *dl1, *dl2, *s2, *zd1, *zd2, *sp2;
    } f{};
    struct {
        __nv_bfloat16 *x, *xd, *ax, *h1, *hd1, *ah1, *dl1, *dl2, *dp1, *dp2;
    } b{};
    float *z3 = nullptr, *out = nullptr, *dl3 = nullptr, *a = nullptr;
    __nv_bfloat16 *w = nullptr;  // BF16 weights of both elements
    float *gw = nullptr;         // weight-gradient products of both elements
    int split = 0;               // 1: every BF16 operand has its low part lo elements further on
    size_t lo = 0;
};
size_t gemm_train_floats(int R);
size_t gemm_train_bf16(int R);  // high parts; the pool holds twice this (low parts after them)
size_t gemm_train_gw(int R);
void gemm_train_carve(GemmTrain &T, float *fpool, __nv_bfloat16 *bpool, float *gw, int R);
int gemm_train_forward(cublasHandle_t h, cudaStream_t s, const GemmTrain &T);
int gemm_train_backward(cublasHandle_t h, cudaStream_t s, const GemmTrain &T);

cudaError_t launch_adam(cudaStream_t s, float *theta, float *m, float *v, const double *grad, int n, double scale,
                        double lr, double b1, double b2, double eps, int step, const uint8_t *frozen);
cudaError_t launch_weights_to_model(cudaStream_t s, const float *theta, float *wf, double *wd, int n);

enum { kPhaseForce = 0, kPhaseProp1 = 1, kPhaseProp2 = 2, kPhaseEnergyOnly = 3 };

}  // namespace mdt
