// mdt_noalloc.cu -- EMT energy and forces for one configuration without any device
// allocation by the library.
//
// Who needs this: code that hands the library device buffers it already owns and may
// not allocate on its own -- for instance a host program whose GPU memory is carved out
// of one pool up front by another runtime, a loop that must never hit the CUDA
// allocator (whose calls can synchronise the device and stall other streams), or a
// caller that has no library context at all.  The regular entry points keep their pair
// scratch in memory the context allocates at batch definition; this one keeps it in a
// file-scope device array instead.
//
// Limits and rules:
//   * at most kNoAllocMaxAtoms = 256 atoms per call (larger configurations are
//     rejected with MDT_ERR_TOO_LARGE); the scratch array is 6 * 256 * 128 doubles =
//     1.5 MiB and stays resident on every GPU that loads the library until the process
//     exits;
//   * every call shares that array: two calls whose kernels overlap on the GPU (on
//     different streams, or from different host threads) race on it and give wrong
//     results; serialise them.  The array keeps the previous call's contents, but every
//     slot a call reads is written by the same call first, so nothing needs clearing;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call before
//     any stream capture begins.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/mdt_gpu.h"
#include "mdt_common.cuh"
#include "mdt_emt.cuh"
#include "mdt_internal.h"

namespace mdt {

// Derived EMT constants of compute_emt_1species / compute_emt_2species
// (src/pes_emt_mod.f90:258-307 and 521-592), in the reference's order of operations; shared
// by mdt_emt_set_params and the allocation-free entry point.  Returns MDT_OK,
// MDT_ERR_UNSUPPORTED (more than two EMT species) or MDT_ERR_ARG (no EMT species).
int emt_derive_constants(int32_t ntypes, const double *eta2, const double *n0, const double *e0, const double *lambda,
                  const double *v0, const double *kappa, const double *s0, const int32_t *pes, EmtConst &E) {
    E = EmtConst{};
    int slots[2] = {-1, -1}, ns = 0;
    for (int t = 0; t < kMaxTypes; ++t) E.slot_of_type[t] = -1;
    for (int t = 0; t < ntypes; ++t)
        if (pes[t * ntypes + t] == MDT_PES_EMT) {
            if (ns >= 2) return MDT_ERR_UNSUPPORTED;
            slots[ns] = t;
            E.slot_of_type[t] = ns++;
        }
    if (ns == 0) return MDT_ERR_ARG;
    E.nspecies = ns;
    for (int a = 0; a < ntypes; ++a)
        for (int b = 0; b < ntypes; ++b)
            if (pes[b * ntypes + a] == MDT_PES_EMT && E.slot_of_type[a] >= 0 && E.slot_of_type[b] >= 0)
                E.pair_mask |= 1u << (a * kMaxTypes + b);
    const double beta = std::pow(16.0 * kPi / 3.0, 1.0 / 3.0) * (1.0 / kSqrt2);
    const double nneighs[3] = {12.0, 6.0, 24.0};
    double bs0[2] = {0, 0};
    for (int s = 0; s < ns; ++s) {
        const int t = slots[s];
        E.eta2[s] = eta2[t];
        E.n0[s] = n0[t];
        E.e0[s] = e0[t];
        E.lambda[s] = lambda[t];
        E.kappa[s] = kappa[t];
        E.v0[s] = v0[t];
        bs0[s] = beta * s0[t];
        E.betas0[s] = bs0[s];
        E.betaeta2[s] = beta * eta2[t];
        E.kappadbeta[s] = kappa[t] / beta;
    }
    const double rcut = (ns == 2 ? std::max(bs0[0], bs0[1]) : bs0[0]) * kSqrt3;
    const double rr = 4.0 * rcut / (kSqrt3 + 2);
    const double acut = 9.21034037197618 / (rr - rcut);
    E.rcut = rcut;
    E.acut = acut;
    E.cut = 1.5 * rcut;
    E.cut2 = E.cut * E.cut;
    for (int s = 0; s < ns; ++s) {
        const double rnn[3] = {bs0[s], bs0[s] * kSqrt2, bs0[s] * kSqrt3};
        double x[3], g1 = 0, g2 = 0;
        for (int k = 0; k < 3; ++k) x[k] = nneighs[k] * kTwelfth / (1 + std::exp(acut * (rnn[k] - rcut)));
        for (int k = 0; k < 3; ++k) g1 += x[k] * std::exp(-E.eta2[s] * (rnn[k] - bs0[s]));
        for (int k = 0; k < 3; ++k) g2 += x[k] * std::exp(-E.kappadbeta[s] * (rnn[k] - bs0[s]));
        E.igamma1[s] = 1.0 / g1;
        E.g2v0[s] = (1.0 / g2) * E.v0[s];
        E.dens_exp[s] = 0.5 / kBohr2Ang - E.betaeta2[s];
    }
    E.chi[0][0] = E.chi[1][1] = 1.0;
    E.chi[0][1] = E.chi[1][0] = 1.0;
    if (ns == 2) {
        const int t1 = slots[0], t2 = slots[1];
        const double chi_21 = n0[t1] / n0[t2] * std::exp(0.5 / kBohr2Ang * (s0[t2] - s0[t1]));
        E.chi[0][1] = 1.0 / chi_21;
        E.chi[1][0] = chi_21;
        E.hh_quirk = 1;
    }
    return MDT_OK;
}

namespace {

constexpr int kNoAllocMaxAtoms = 256;
constexpr size_t kNoAllocScratch = 6 * (size_t)kNoAllocMaxAtoms * (kNoAllocMaxAtoms / 2);

static __device__ __align__(256) double g_noalloc_pair_scratch[kNoAllocScratch];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {nullptr};

// invert_matrix, src/useful_things.f90:296-321 (column major), as mdt_batch_define does
bool invert_cell(const double *A, double *B) {
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

struct CellArg {
    double h[9], hi[9];
};

constexpr int kNoAllocBlock = 128;

// One CTA evaluates the configuration with the same device function as the context
// path (emt_bead), pointed at caller buffers and the file-scope scratch.
__global__ void __launch_bounds__(kNoAllocBlock) emt_noalloc_kernel(int N, int ntypes, CellArg cell, EmtConst E,
                                                                     const double *x,
                                                                     const double *y, const double *z,
                                                                     const int32_t *idx, double *fx, double *fy,
                                                                     double *fz, double *energy, double *dens,
                                                                     double *scratch) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_natoms, s_nbeads, s_zero;
    __shared__ int64_t s_zero64;
    __shared__ double s_box[9], s_ibox[9];
    __shared__ int s_bad;
    int8_t *s_type = (int8_t *)smem_raw;
    double *s_dens = (double *)(smem_raw + ((N + 15) & ~15));
    unsigned char *emt_base = smem_raw + ((N + 15) & ~15) + ((8 * (size_t)N + 15) & ~size_t(15));
    if (threadIdx.x == 0) {
        s_natoms = N;
        s_nbeads = 1;
        s_zero = 0;
        s_zero64 = 0;
        s_bad = 0;
        *energy = 0.0;
    }
    if (threadIdx.x < 9) {
        s_box[threadIdx.x] = cell.h[threadIdx.x];
        s_ibox[threadIdx.x] = cell.hi[threadIdx.x];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        int ty = idx[i] - 1;
        if (ty < 0 || ty >= ntypes) {  // a type outside the parameter table
            s_bad = 1;
            ty = 0;
        }
        s_type[i] = (int8_t)ty;
        fx[i] = 0.0;
        fy[i] = 0.0;
        fz[i] = 0.0;
    }
    __syncthreads();
    Batch B{};
    B.ntraj = 1;
    B.natoms = &s_natoms;
    B.nbeads = &s_nbeads;
    B.ba_off = &s_zero64;
    B.atom_off = &s_zero;
    B.bead_off = &s_zero;
    B.pair_off = &s_zero64;
    B.rx = const_cast<double *>(x);
    B.ry = const_cast<double *>(y);
    B.rz = const_cast<double *>(z);
    B.fx = fx;
    B.fy = fy;
    B.fz = fz;
    B.dens = dens ? dens : s_dens;
    B.epot = energy;
    B.type = s_type;
    B.box = s_box;
    B.ibox = s_ibox;
    B.pair_scratch = scratch;
    B.max_atoms = N;
    B.max_beads = 1;
    SmemEmt<double> S = carve_smem<double>(emt_base, N, 1);
    emt_bead<double>(B, E, S, 0, 0, true);
    if (threadIdx.x == 0 && s_bad) *energy = NAN;
}

}  // namespace
}  // namespace mdt

using namespace mdt;

extern "C" int32_t mdt_emt_force_noalloc(int32_t natoms, const int32_t *idx, const double *x, const double *y,
                                         const double *z, const double *simbox, int32_t ntypes, const double *eta2,
                                         const double *n0, const double *e0, const double *lambda,
                                         const double *v0, const double *kappa, const double *s0,
                                         const int32_t *pes, double *fx, double *fy, double *fz, double *energy,
                                         double *dens, void *stream) {
    if (natoms > kNoAllocMaxAtoms) return MDT_ERR_TOO_LARGE;
    if (natoms < 1 || !idx || !x || !y || !z || !simbox || !fx || !fy || !fz || !energy || ntypes < 1 ||
        ntypes > kMaxTypes || !eta2 || !n0 || !e0 || !lambda || !v0 || !kappa || !s0 || !pes)
        return MDT_ERR_ARG;
    EmtConst E;
    int rc = emt_derive_constants(ntypes, eta2, n0, e0, lambda, v0, kappa, s0, pes, E);
    if (rc != MDT_OK) return rc;
    CellArg cell;
    for (int k = 0; k < 9; ++k) cell.h[k] = simbox[k];
    if (!invert_cell(cell.h, cell.hi)) return MDT_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MDT_ERR_CUDA;
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_pair_scratch) != cudaSuccess) return MDT_ERR_CUDA;
            g_scratch_addr[dev] = (double *)p;
        }
        scratch = g_scratch_addr[dev];
    }
    const size_t sm = ((natoms + 15) & ~15) + ((8 * (size_t)natoms + 15) & ~size_t(15)) + smem_bytes(natoms, 1, 8);
    emt_noalloc_kernel<<<1, kNoAllocBlock, sm, (cudaStream_t)stream>>>(natoms, ntypes, cell, E, x, y, z, idx, fx, fy, fz,
                                                                       energy, dens, scratch);
    return cudaGetLastError() == cudaSuccess ? MDT_OK : MDT_ERR_CUDA;
}
