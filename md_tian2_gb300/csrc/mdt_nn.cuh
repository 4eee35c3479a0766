// mdt_nn.cuh -- atom-centred symmetry functions (G2/G3), per-element MLP and analytic
// forces for one bead inside a CTA: the RuNNer short-range prediction of md_tian2's
// compute_nene (src/pes_nene_mod.f90:7145-7368), restated for the GPU.
//
//   neighbour list  thread per atom, in RuNNer's order i -> j -> n1 -> n2 -> n3
//                   (RuNNer_src/neighbor_para_short.f90:117-163), packed (j, image)
//                   words in a global scratch slot per bead-atom;
//   descriptors     warp per central atom: the neighbour cache (relative vector,
//                   distance, cutoff value/derivative, exp(-eta r^2) per distinct G3 eta)
//                   sits in the warp's shared memory, lanes stride over the first
//                   neighbour j of a triplet and loop over k > j, so the triplet term
//                   needs no transcendental beyond exp(-eta r_jk^2) and the r_jk cutoff;
//   network         lanes are the nodes of a layer (weights in shared memory);
//   forces          reverse mode: dE/dG from the network, then a second walk over the
//                   same pairs/triplets scatters dE/dG . dG/dx into per-slot force
//                   accumulators (RuNNer builds dG/dx explicitly and contracts it
//                   forward-mode, RuNNer_src/getshortatomic.f90:263-322; both give the
//                   same forces).
#pragma once
#include "mdt_common.cuh"

namespace mdt {

constexpr int kMaxElem = 4;
constexpr int kMaxSF = 64;
constexpr int kMaxNodes = 64;
constexpr int kMaxLayers = 4;
constexpr int kMaxEta = 6;
constexpr int kNNWarps = 4;  // warps (central atoms in flight) per CTA

struct NNDev {
    int nelem, maxsf, nlayers, maxnodes, maxweights, maxnb;
    int elem_of_type[kMaxTypes];  // universe type -> element index (-1: not NN)
    int cutoff_type;
    double cutoff_alpha;
    int scalesym, centersym, normnodes, remove_atom_energies;
    double scmin, scmax;
    double rc[kMaxElem];          // cutoff shared by all symmetry functions of an element (bohr)
    double maxcut;                // neighbour-list cutoff (bohr)
    int ng3eta[kMaxElem];
    double g3eta[kMaxElem][kMaxEta];
    int nsf[kMaxElem];
    int nodes[kMaxElem][kMaxLayers + 1];
    int woff[kMaxElem][kMaxLayers + 1];  // offset of each layer's weights
    // per element e and symmetry function s at [e*maxsf + s]
    const int *sftype, *e1, *e2, *izeta, *etaslot;
    const double *eta, *rs, *lam, *zeta, *pnorm, *smin, *smax, *savg;
    const uint8_t *act;           // [e][layer][node]
    const double *wd;             // weights, FP64
    const float *wf;              // weights, FP32 copy
    double atom_energy[kMaxElem]; // Ha
    float margin;                 // descriptor range margin (fraction of max-min) for the fallback
    // G3 "grid" form: every G3 function of the element is one (eta slot m, (lambda,zeta)
    // slot q) cell and all share one neighbour-element pair; then the per-triplet work
    // is an outer product of ng exponentials with nlz angular powers held in registers.
    int g3fast[kMaxElem];
    int nlz[kMaxElem];
    float lz_lam[kMaxElem][8], lz_zl[kMaxElem][8], lz_pnorm[kMaxElem][8];
    int lz_zm1[kMaxElem][8];             // zeta - 1 (integer)
    int8_t sf_of[kMaxElem][4][8];        // symmetry-function index of cell (m, q), -1 if none
    int g3pair[kMaxElem][2];             // the shared neighbour-element pair
};

// ---------------------------------------------------------------------------
// FP32 fast path (mdt_nnf.cu).  Applies when every symmetry function is a radial G2
// or a narrow angular G3 with one cosine cutoff (alpha = 0) shared by all functions,
// and the G3 functions of each element form a grid of eta slots x (lambda = +-1,
// zeta = 2^b) cells over one neighbour-element pair.
// ---------------------------------------------------------------------------
constexpr int kFMaxG2 = 24;  // radial functions per element
constexpr int kFNQ = 8;      // (lambda, zeta) cells: lambda = +-1 for up to 4 zeta values

struct FastNN {
    int ok;                        // model qualifies
    int ng, zm;                    // eta slots; zeta mask (bit b set: zeta = 2^b is used)
    int anyg3;                     // some element has G3 functions
    float rc2, inv_rc2;            // bohr^-2
    float cut2_hi, cut2_lo;        // FP32 screen of the neighbour list (bohr^2)
    float skin, cut2s;             // Verlet skin (bohr, 0: off) and the skin list's squared cutoff
    int hasg3[kMaxElem];
    int pair_a[kMaxElem], pair_b[kMaxElem];  // G3 neighbour-element pair (element indices)
    float g3l2[kMaxElem][4];       // -eta_m log2(e), for exp2
    float g3eta[kMaxElem][4];      // eta_m
    int8_t cell_sf[kMaxElem][4][kFNQ];  // SF index of cell (m, 2k + [lambda < 0]), -1 if none
    float cell_lz[kFNQ];           // lambda zeta of cell q
    int ng2[kMaxElem];
    // radial functions of element e: g2tab[e*kFMaxG2 + k], k < ng2[e], ordered by neighbour element
    const float4 *g2tab;           // (-eta log2 e, r_s, -2 eta, sf index | neighbour element << 8)
    // network weights as the fast kernels keep them in shared memory: layer l of element
    // e is a row-major (n_{l-1} + 1) x stride matrix (last row: biases) at wofs[e][l]
    int wofs[kMaxElem][kMaxLayers + 1], wstr[kMaxElem][kMaxLayers + 1], wtotal;
    const float4 *scal;            // [e*maxsf + s]: scaled = x g + y; outside [z, w] raises the flag
    const float *dscal;            // [e*maxsf + s]: d(scaled)/dG as RuNNer applies it
};

// ---------------------------------------------------------------------------
// FP32 thread-per-atom kernel of radial-only models (mdt_nnr.cu).  Applies when every
// symmetry function is a G2 under one cosine cutoff, there are at most two elements,
// every centre element has the same (eta, r_s) list per neighbour element, and the
// network has one or two hidden layers of at most 32 nodes with one activation per
// layer.  Descriptors live in a padded grouped order: slots [0, ka) are the functions
// over neighbour element 0, [ka, ka + kb) those over element 1.
// ---------------------------------------------------------------------------
constexpr int kRBlockMax = 512;  // threads per CTA (atoms of a pack)
constexpr int kRMaxTraj = 32;    // trajectories per pack
constexpr int kRMaxK = 24;       // functions per neighbour element

// Shared-memory layout constants of a shape (nin = functions per atom, nh = hidden
// layers): weight block of one element (W1 + b1, then W2, b2, W2T, w3, b3 + 3 pad or
// w2, b2 + 3 pad), offset of element 1's block (64 bytes off the 128-byte grid), both
// blocks, per-thread buffer floats (two hidden layers: layer-1 values and delta2 side by
// side).
__host__ __device__ constexpr int nnr_wblock(int nin, int nh) {
    return 32 * (nin + 1) + (nh == 2 ? 2 * 32 * 32 + 2 * 32 + 4 : 32 + 4);
}
__host__ __device__ constexpr int nnr_wofs1(int nin, int nh) { return ((nnr_wblock(nin, nh) + 31) & ~31) + 16; }
__host__ __device__ constexpr int nnr_wtotal(int nin, int nh) { return nnr_wofs1(nin, nh) + nnr_wblock(nin, nh); }
__host__ __device__ constexpr int nnr_hbw(int nin, int nh) {
    return nin > (nh == 2 ? 64 : 32) ? nin : (nh == 2 ? 64 : 32);
}

// Tensor-core (BF16 in, FP32 accumulate) network of the same kernel: the atoms of a CTA
// are four 128-row tiles; per tile and layer one GEMM (M = 128) runs on tcgen05 with the
// operand rows in shared memory and the accumulator in TMEM.  Inputs are padded to a
// multiple of 16 (KP), hidden layers to 32; the operand buffer of a tile holds rows of
// TW = max(KP, 32) bf16 values.  Per element the B operands are W1^T (32 x KP), W2^T and
// W2 (32 x 32) and W1 (KP x 32), K-major; biases and the output weights stay FP32.
__host__ __device__ constexpr int nnr_kp(int nin) { return (nin + 15) & ~15; }
__host__ __device__ constexpr int nnr_tw(int nin) { return nnr_kp(nin) > 32 ? nnr_kp(nin) : 32; }
__host__ __device__ constexpr int nnr_tc_bel(int nin) { return 2 * (32 * nnr_kp(nin) * 2) + 2 * 2048; }
constexpr int kTcVec = 100;          // FP32 vector floats per element (b1, b2 / w2, w3, b3, pad)
constexpr int kTcTiles = kRBlockMax / 128;
constexpr int kTcCols = 512;         // TMEM columns of a CTA (D of both elements + a spill, per tile)
constexpr size_t kTcEmtMin = 36864;  // the operand area doubles as the FP64 EMT fallback area
__host__ __device__ constexpr size_t nnr_tc_hb(int nin) {
    return (size_t)kTcTiles * 128 * nnr_tw(nin) * 2 > kTcEmtMin ? (size_t)kTcTiles * 128 * nnr_tw(nin) * 2
                                                                  : kTcEmtMin;
}
__host__ __device__ constexpr int nnr_tc_cpt(int nin) { return 2 * nnr_tw(nin) + 32; }
static_assert(kTcTiles * nnr_tc_cpt(48) <= kTcCols, "TMEM columns of the widest shape");

struct RadialNN {
    int ok;
    int ka, kb, nh;                 // kernel shape: padded functions per group, hidden layers
    int bla, blb;                   // recurrence block length per group (0: one 2^x per function)
    int nelem, nin;                 // elements, ka + kb
    int block;                      // threads per CTA (batch plan)
    int surrogate, maxnb;
    int elem_of_type[kMaxTypes];
    float rc2, inv_rc2, rc_b, rcs;  // cutoff^2, 1/cutoff^2, cutoff, skin-list cutoff (bohr)
    float skin, cut2s;              // Verlet skin (bohr, 0: off), skin-list cutoff^2 (bohr^2)
    float c[2][kRMaxK];             // -eta log2(e) (bohr^-2); 0 on padded slots
    float rs[2][kRMaxK];            // r_s (bohr)
    // recurrence of a group with one eta and r_s spaced by delta: the ratio of consecutive
    // functions is q = 2^(gq u + gc) (u = r - r_s), and consecutive q differ by gam
    float gq[2], gc[2], gam[2], dl[2];
    uint8_t act[3];                 // activation of hidden layers 1..nh, then of the output
    float rn[3];                    // 1/n_(l-1) per layer with normnodes, else 1
    double atom_energy[2];          // Ha (0 unless remove_atom_energies)
    // weight blocks in shared memory (nnr_wblock layout), built from the model's FP32
    // weights at kernel start
    const float *wf;                // model weights (NNDev::wf layout)
    int maxweights, woff[2][kMaxLayers + 1], nodes[2][kMaxLayers + 1];
    int8_t qsrc[2][2 * kRMaxK];     // model descriptor index of padded slot q (-1: none)
    const float4 *fscal;            // FastNN::scal / dscal (model order), permuted at kernel start
    const float *fdscal;
    int maxsf;
    int tc;                         // 1: network GEMMs on the tensor cores (BF16 operands)
};

// ---------------------------------------------------------------------------
// Host-visible launch parameters of the NN kernels
// ---------------------------------------------------------------------------
struct NNScratch {
    int *nbw;          // packed neighbour words, [ba][maxnb]
    int *nbcnt;        // neighbour count per bead-atom
    const int *img;    // per trajectory 3 image counts (na, nb, nc)
    int *fallback;     // per trajectory: beads that fell back to EMT (surrogate)
    int *nnstatus;     // per trajectory: 1 = neighbour list overflow
    double *gout;      // optional: raw symmetry functions [ba][maxsf] (descriptor export)
    unsigned *mscr;    // fast path: triplet masks of a bead, mcap words per CTA
    int mcap;
    // fast path Verlet skin lists: per bead-atom skcap entries (j, packed unwrapped image),
    // count (-1: overflow, full build), reference positions, per-bead validity
    int2 *skw;
    int *skcnt;
    double *skref;
    int *skok;
    int skcap;
    int *tcerr;        // set when a tensor-core GEMM did not complete within its wait limit
    const double *lcoef;  // thread-per-atom kernel: constant-friction Langevin coefficients, 8 per slot
    // generic kernels: dE/dG [ba][maxsf] and the atomic energies (Ha, output node) of a prior
    // tensor-core network pass; when set, the kernels skip descriptors and network and run the
    // forces (descriptor VJP) from them
    const float *dgin;
    const double *eatin;
};

// ---------------------------------------------------------------------------
template <typename R> struct NM;
template <> struct NM<double> {
    static __device__ __forceinline__ double ex(double x) { return exp(x); }
    static __device__ __forceinline__ double sq(double x) { return sqrt(x); }
    static __device__ __forceinline__ void sc(double x, double *s, double *c) { sincospi(x, s, c); }
    static __device__ __forceinline__ double th(double x) { return tanh(x); }
    static __device__ __forceinline__ double lg(double x) { return log(x); }
    static __device__ __forceinline__ double pw(double a, double b) { return pow(a, b); }
    static __device__ __forceinline__ const double *w(const NNDev &M) { return M.wd; }
};
template <> struct NM<float> {
    static __device__ __forceinline__ float ex(float x) { return __expf(x); }
    static __device__ __forceinline__ float sq(float x) { return sqrtf(x); }
    static __device__ __forceinline__ void sc(float x, float *s, float *c) { sincospif(x, s, c); }
    static __device__ __forceinline__ float th(float x) { return tanhf(x); }
    static __device__ __forceinline__ float lg(float x) { return __logf(x); }
    static __device__ __forceinline__ float pw(float a, float b) { return powf(a, b); }
    static __device__ __forceinline__ const float *w(const NNDev &M) { return M.wf; }
};

// cutoff function and derivative, RuNNer_src/getcutoff.f90:51-162
template <typename R>
__device__ __forceinline__ void cutoff_fn(const NNDev &M, R rc, R r, R &fc, R &dfc) {
    const R rci = (R)M.cutoff_alpha * rc, iw = R(1) / (rc - rci);
    const int type = M.cutoff_type;
    if (type == 0) { fc = R(1); dfc = R(0); return; }
    if (type == 1) {
        if (r <= rci) { fc = R(1); dfc = R(0); return; }
        const R x = (r - rci) * iw;
        R s, c;
        NM<R>::sc(x, &s, &c);
        fc = R(0.5) * (c + R(1));
        dfc = -s * (R(kPi) / R(2)) * iw;
        return;
    }
    if (type == 2 || type == 3) {
        const R pref = type == 3 ? (R)(((2.718281828459045 + 1.0) / (2.718281828459045 - 1.0)) *
                                       ((2.718281828459045 + 1.0) / (2.718281828459045 - 1.0)) *
                                       ((2.718281828459045 + 1.0) / (2.718281828459045 - 1.0)))
                                 : R(1);
        if (r <= rci) {
            const R t = NM<R>::th(R(1));
            fc = pref * t * t * t;
            dfc = R(0);
            return;
        }
        const R t = NM<R>::th(R(1) - r / rc);
        fc = pref * t * t * t;
        dfc = pref * (R(-3) / rc) * (t * t - t * t * t * t);
        return;
    }
    if (r <= rci) { fc = R(1); dfc = R(0); return; }
    const R x = (r - rci) * iw;
    if (type == 4) {
        const R q = R(1) - x * x;
        fc = NM<R>::ex(R(1) - R(1) / q);
        dfc = (R(-2) * iw * x / (q * q)) * fc;
    } else if (type == 5) {
        fc = (R(2) * x - R(3)) * x * x + R(1);
        dfc = iw * x * (R(6) * x - R(6));
    } else if (type == 6) {
        fc = ((R(15) - R(6) * x) * x - R(10)) * x * x * x + R(1);
        dfc = iw * x * x * ((R(60) - R(30) * x) * x - R(30));
    } else if (type == 7) {
        fc = (x * (x * (R(20) * x - R(70)) + R(84)) - R(35)) * x * x * x * x + R(1);
        dfc = x * x * x * iw * (x * (x * (R(140) * x - R(420)) + R(420)) - R(140));
    } else {
        const R x4 = x * x * x * x;
        fc = (x * (x * (x * (R(315) - R(70) * x) - R(540)) + R(420)) - R(126)) * x4 * x + R(1);
        dfc = iw * x4 * (x * (x * ((R(2520) - R(630) * x) * x - R(3780)) + R(2520)) - R(630));
    }
}

// activation and derivative, RuNNer_src/calconenn.f90:124-146, getdnodes_values.f90:76-108
template <typename R> __device__ __forceinline__ R act_fn(uint8_t a, R x) {
    switch (a) {
        case 't': return NM<R>::th(x);
        case 'g': return NM<R>::ex(R(-0.5) * x * x);
        case 'c': return cos(x);
        case 's': return R(1) / (R(1) + NM<R>::ex(-x));
        case 'S': return R(1) - R(1) / (R(1) + NM<R>::ex(-x));
        case 'e': return NM<R>::ex(-x);
        case 'p': return NM<R>::lg(NM<R>::ex(x) + R(1));
        case 'h': return x * x;
        default: return x;  // 'l'
    }
}
template <typename R> __device__ __forceinline__ R act_dfn(uint8_t a, R sum, R val) {
    switch (a) {
        case 't': return R(1) - val * val;
        case 'g': return R(-1) * sum * val;
        case 'c': return -sin(sum);
        case 's': { const R e = NM<R>::ex(-sum); return e / ((R(1) + e) * (R(1) + e)); }
        case 'S': { const R e = NM<R>::ex(-sum); return -e / ((R(1) + e) * (R(1) + e)); }
        case 'e': return -val;
        case 'p': { const R e = NM<R>::ex(val); return (e - R(1)) / e; }
        case 'h': return R(2) * sum;
        default: return R(1);
    }
}

// second derivative of the activation (used by the force-loss training gradient)
template <typename R> __device__ __forceinline__ R act_ddfn(uint8_t a, R sum, R val) {
    switch (a) {
        case 't': return R(-2) * val * (R(1) - val * val);
        case 'p': { const R e = NM<R>::ex(-sum); const R s = R(1) / (R(1) + e); return s * (R(1) - s); }
        case 's': { const R s = val; return s * (R(1) - s) * (R(1) - R(2) * s); }
        case 'g': return (sum * sum - R(1)) * val;
        case 'e': return val;
        case 'h': return R(2);
        default: return R(0);
    }
}

// Integer power by squaring (G3 (1 + lambda cos)^(zeta-1) for integer zeta).
template <typename R> __device__ __forceinline__ R ipow(R x, int n) {
    R r = R(1);
    while (n > 0) {
        if (n & 1) r *= x;
        x *= x;
        n >>= 1;
    }
    return r;
}

}  // namespace mdt
