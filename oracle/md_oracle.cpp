/*
 * md_oracle.cpp -- CPU FP64 restatement of md_tian2's force evaluation and
 * propagators.  TEST INFRASTRUCTURE ONLY (see md_oracle.h): the checker for the
 * CUDA engine and the timed CPU baseline; never part of the product path.
 *
 * Every routine follows the reference's Fortran expression by expression and in the
 * same loop order, including its dense (3,nb,N,N) derivative tensors, so that the
 * operation count of the CPU baseline matches the reference's.  Reference quirks are
 * kept on purpose and marked "QUIRK".
 * Parity: unpinned by a reference run (no Fortran compiler); see md_oracle.h.
 */
#include "md_oracle.h"

#include <algorithm>
#include <chrono>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

// src/constants.f90:30-39,157-170
const double kPi = 3.14159265358979323846264338327950288;
const double kSqrt2 = 1.41421356237309504880168872420969808;
const double kSqrt3 = 1.73205080756887729352744634150587237;
const double kIsqrt2 = 1.0 / kSqrt2;
const double kB = 8.61733238496e-5;
const double kHbar = 0.6582119514467406;
const double kTwelfth = 1.0 / 12.0;
const double kTolerance = 1.0e-9;
const double kBohr2Ang = 0.529177211;
const double kAmu2Mass = 103.638239276;
const int kPesEmt = 2003;

// Single-precision literals the reference mixes into double expressions.
const double kF1em30 = (double)1e-30f;   // pes_emt_mod.f90:382,793-794
const double kF1em2 = (double)1e-2f;     // md_algo.f90:176,264
const double kF036 = (double)0.36f;      // md_algo.f90:542,549
const double kFm1em12 = (double)-1e-12f; // md_algo.f90:542

inline size_t I3(int d, int b, int i, int nb) { return ((size_t)i * nb + b) * 3 + d; }
inline size_t I2(int b, int i, int nb) { return (size_t)i * nb + b; }
inline size_t I4(int d, int b, int i, int j, int nb, int n) {
    return (((size_t)j * n + i) * nb + b) * 3 + d;
}

enum { P_ETA2 = 0, P_N0, P_E0, P_LAMBDA, P_V0, P_KAPPA, P_S0 };
inline double par(const orc_universe *u, int type1based, int k) {
    return u->emt[(type1based - 1) * 7 + k];
}
inline int pes_of(const orc_universe *u, int t1, int t2) {
    return u->pes[(t2 - 1) * u->ntypes + (t1 - 1)];
}

// select_beta('fcc'), pes_emt_mod.f90:1664-1677
double select_beta_fcc() { return std::pow(16.0 * kPi / 3.0, 1.0 / 3.0) * kIsqrt2; }

// Fortran anint: round half away from zero
inline double anint(double x) { return std::round(x); }

// ---------------------------------------------------------------------------
// compute_emt_1species, pes_emt_mod.f90:230-477
// ---------------------------------------------------------------------------
void emt_1species(orc_universe *u, const double *distances, const double *vectors) {
    const int N = u->natoms, nb = u->nbeads;
    const double cutoff = 1.5;
    int emt_idx = 0;
    for (int i = 1; i <= u->ntypes; ++i)
        if (pes_of(u, i, i) == kPesEmt) emt_idx = i;

    const double beta = select_beta_fcc();
    const double nneighs[3] = {12.0, 6.0, 24.0};
    const double betas0 = beta * par(u, emt_idx, P_S0);
    const double betaeta2 = beta * par(u, emt_idx, P_ETA2);
    const double kappadbeta = par(u, emt_idx, P_KAPPA) / beta;
    double rnn[3] = {betas0, betas0 * kSqrt2, betas0 * kSqrt3};
    const double rcut = betas0 * kSqrt3;
    const double rr = 4.0 * rcut / (kSqrt3 + 2);
    const double acut = 9.21034037197618 / (rr - rcut);
    double x[3], r3temp[3];
    for (int k = 0; k < 3; ++k) x[k] = nneighs[k] * kTwelfth / (1 + std::exp(acut * (rnn[k] - rcut)));
    for (int k = 0; k < 3; ++k) r3temp[k] = rnn[k] - betas0;
    double s1 = 0, s2 = 0;
    for (int k = 0; k < 3; ++k) s1 += x[k] * std::exp(-par(u, emt_idx, P_ETA2) * r3temp[k]);
    for (int k = 0; k < 3; ++k) s2 += x[k] * std::exp(-kappadbeta * r3temp[k]);
    const double igamma1 = 1.0 / s1, igamma2 = 1.0 / s2;

    std::vector<double> V(nb, 0.0), Ecoh(nb, 0.0), vref(nb, 0.0), rtemp_beads(nb);
    std::vector<double> s(nb * N, 0.0), exp_lambda_s(nb * N, 0.0), sigma(nb * N, 0.0);
    std::vector<double> dV(3 * nb * N, 0.0), dEcoh(3 * nb * N, 0.0), dvref(3 * nb * N, 0.0);
    std::vector<double> dsigma(3 * (size_t)nb * N * N, 0.0), ds(3 * (size_t)nb * N * N, 0.0);

    for (int i = 0; i < N - 1; ++i) {
        const int idx_i = u->idx[i];
        for (int j = i + 1; j < N; ++j) {
            const int idx_j = u->idx[j];
            if (pes_of(u, idx_i, idx_j) != kPesEmt) continue;
            for (int b = 0; b < nb; ++b) {
                const double rijmag = distances[((size_t)j * N + i) * nb + b];
                const double *rij = &vectors[I4(0, b, i, j, nb, N)];
                if (rijmag > cutoff * rcut) continue;
                double rtemp = std::exp(acut * (rijmag - rcut));
                const double theta = 1.0 / (1 + rtemp);
                const double rtemp1 = acut * rtemp * theta;
                rtemp = theta * std::exp(-par(u, emt_idx, P_ETA2) * (rijmag - betas0));
                sigma[I2(b, i, nb)] += rtemp;
                sigma[I2(b, j, nb)] += rtemp;
                for (int d = 0; d < 3; ++d) {
                    const double dtheta = (par(u, emt_idx, P_ETA2) + rtemp1) * rtemp * rij[d] / rijmag;
                    dsigma[I4(d, b, i, i, nb, N)] -= dtheta;
                    dsigma[I4(d, b, j, j, nb, N)] += dtheta;
                    dsigma[I4(d, b, j, i, nb, N)] = dtheta;
                    dsigma[I4(d, b, i, j, nb, N)] = -dtheta;
                }
                rtemp = theta * std::exp(-kappadbeta * (rijmag - betas0));
                V[b] += rtemp;
                for (int d = 0; d < 3; ++d) {
                    const double dtheta = (kappadbeta + rtemp1) * rtemp * rij[d] / rijmag;
                    dV[I3(d, b, i, nb)] += dtheta;
                    dV[I3(d, b, j, nb)] -= dtheta;
                }
            }
        }
    }
    const double v0 = par(u, emt_idx, P_V0);
    for (auto &q : sigma) q *= igamma1;
    for (auto &q : V) q = q * igamma2 * v0;
    for (auto &q : dsigma) q *= igamma1;
    for (auto &q : dV) q = q * igamma2 * v0;

    for (size_t k = 0; k < s.size(); ++k) s[k] = std::max(kF1em30, sigma[k]);
    for (size_t k = 0; k < ds.size(); ++k) ds[k] = -dsigma[k];
    for (int i = 0; i < N; ++i) {
        const int idx_i = u->idx[i];
        for (int j = 0; j < N; ++j) {
            const int idx_j = u->idx[j];
            if (pes_of(u, idx_i, idx_j) == kPesEmt)
                for (int b = 0; b < nb; ++b)
                    for (int d = 0; d < 3; ++d)
                        ds[I4(d, b, i, j, nb, N)] = ds[I4(d, b, i, j, nb, N)] / (betaeta2 * s[I2(b, j, nb)]);
        }
    }
    for (auto &q : s) q = -std::log(std::max(kTolerance, q) * kTwelfth) / betaeta2;

    const double rtemp1 = 0.5 / kBohr2Ang - betaeta2;
    for (int i = 0; i < N; ++i) {
        const int idx_i = u->idx[i];
        if (pes_of(u, idx_i, idx_i) == kPesEmt) {
            for (int b = 0; b < nb; ++b) {
                const double si = s[I2(b, i, nb)];
                u->dens[I2(b, i, nb)] = par(u, idx_i, P_N0) * std::exp(rtemp1 * si);
                exp_lambda_s[I2(b, i, nb)] = std::exp(-par(u, idx_i, P_LAMBDA) * si);
                Ecoh[b] += ((1 + par(u, idx_i, P_LAMBDA) * si) * exp_lambda_s[I2(b, i, nb)] - 1);
            }
        }
    }
    for (auto &q : Ecoh) q *= par(u, emt_idx, P_E0);

    for (int i = 0; i < N; ++i) {
        const int idx_i = u->idx[i];
        for (int j = 0; j < N; ++j) {
            const int idx_j = u->idx[j];
            if (pes_of(u, idx_i, idx_j) == kPesEmt)
                for (int b = 0; b < nb; ++b)
                    for (int d = 0; d < 3; ++d)
                        dEcoh[I3(d, b, i, nb)] += s[I2(b, j, nb)] * exp_lambda_s[I2(b, j, nb)] *
                                                  ds[I4(d, b, i, j, nb, N)];
        }
    }
    {
        const double c = par(u, emt_idx, P_E0) * par(u, emt_idx, P_LAMBDA) * par(u, emt_idx, P_LAMBDA);
        for (auto &q : dEcoh) q = c * q;
    }

    for (int i = 0; i < N; ++i) {
        if (u->idx[i] == emt_idx) {
            for (int b = 0; b < nb; ++b) {
                rtemp_beads[b] = std::exp(-par(u, emt_idx, P_KAPPA) * s[I2(b, i, nb)]);
                vref[b] += rtemp_beads[b];
            }
            for (int j = 0; j < N; ++j)
                if (u->idx[j] == emt_idx)
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dvref[I3(d, b, j, nb)] += rtemp_beads[b] * ds[I4(d, b, j, i, nb, N)];
        }
    }
    {
        const double rtemp = 12 * v0;
        for (auto &q : vref) q *= rtemp;
        for (auto &q : dvref) q = q * rtemp * par(u, emt_idx, P_KAPPA);
    }
    for (int b = 0; b < nb; ++b) u->epot[b] = u->epot[b] + Ecoh[b] - V[b] + 0.5 * vref[b];
    for (int i = 0; i < N; ++i)
        if (u->idx[i] == emt_idx)
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d)
                    u->f[I3(d, b, i, nb)] = u->f[I3(d, b, i, nb)] + dEcoh[I3(d, b, i, nb)] -
                                            dV[I3(d, b, i, nb)] + 0.5 * dvref[I3(d, b, i, nb)];
}

// ---------------------------------------------------------------------------
// compute_emt_2species, pes_emt_mod.f90:483-1027
// ---------------------------------------------------------------------------
void emt_2species(orc_universe *u, const double *distances, const double *vectors) {
    const int N = u->natoms, nb = u->nbeads;
    const size_t n3 = 3 * (size_t)nb * N, n4 = 3 * (size_t)nb * N * N, n2 = (size_t)nb * N;
    const double cutoff = 1.5;
    int type1 = -1, type2 = -1;
    for (int i = 1; i <= u->ntypes; ++i)
        if (pes_of(u, i, i) == kPesEmt) {
            if (type1 < 0) type1 = i;
            else type2 = i;
        }
    const double beta = select_beta_fcc();
    const double nneighs[3] = {12.0, 6.0, 24.0};
    const double betas0_1 = beta * par(u, type1, P_S0), betas0_2 = beta * par(u, type2, P_S0);
    const double betaeta2_1 = beta * par(u, type1, P_ETA2), betaeta2_2 = beta * par(u, type2, P_ETA2);
    const double kappadbeta_1 = par(u, type1, P_KAPPA) / beta, kappadbeta_2 = par(u, type2, P_KAPPA) / beta;
    const double chi_21 = par(u, type1, P_N0) / par(u, type2, P_N0) *
                          std::exp(0.5 / kBohr2Ang * (par(u, type2, P_S0) - par(u, type1, P_S0)));
    const double chi_12 = 1.0 / chi_21;
    const double rnn_1[3] = {betas0_1, betas0_1 * kSqrt2, betas0_1 * kSqrt3};
    const double rnn_2[3] = {betas0_2, betas0_2 * kSqrt2, betas0_2 * kSqrt3};
    const double rcut = std::max(betas0_1, betas0_2) * kSqrt3;
    const double rr = 4.0 * rcut / (kSqrt3 + 2);
    const double acut = 9.21034037197618 / (rr - rcut);
    double x_1[3], x_2[3];
    for (int k = 0; k < 3; ++k) x_1[k] = nneighs[k] * kTwelfth / (1 + std::exp(acut * (rnn_1[k] - rcut)));
    for (int k = 0; k < 3; ++k) x_2[k] = nneighs[k] * kTwelfth / (1 + std::exp(acut * (rnn_2[k] - rcut)));
    double a = 0, bsum = 0;
    for (int k = 0; k < 3; ++k) a += x_1[k] * std::exp(-par(u, type1, P_ETA2) * (rnn_1[k] - betas0_1));
    for (int k = 0; k < 3; ++k) bsum += x_1[k] * std::exp(-kappadbeta_1 * (rnn_1[k] - betas0_1));
    const double igamma1_1 = 1.0 / a, igamma2_1 = 1.0 / bsum;
    a = 0; bsum = 0;
    for (int k = 0; k < 3; ++k) a += x_2[k] * std::exp(-par(u, type2, P_ETA2) * (rnn_2[k] - betas0_2));
    for (int k = 0; k < 3; ++k) bsum += x_2[k] * std::exp(-kappadbeta_2 * (rnn_2[k] - betas0_2));
    const double igamma1_2 = 1.0 / a, igamma2_2 = 1.0 / bsum;

    std::vector<double> V_12(nb, 0), V_21(nb, 0), V_22(nb, 0), V_11(nb, 0), Ecoh_2(nb, 0), Ecoh_1(nb, 0);
    std::vector<double> vref_2(nb, 0), vref_1(nb, 0), rtemp_beads(nb, 0);
    std::vector<double> sigma_22(n2, 0), sigma_21(n2, 0), s_2(n2, 0), sigma_11(n2, 0), sigma_12(n2, 0),
        s_1(n2, 0), exp_lambda_s1(n2, 0), exp_lambda_s2(n2, 0);
    std::vector<double> dsigma_21_2(n3, 0), dsigma_12_1(n3, 0);
    std::vector<double> dEcoh_2_2(n3, 0), dEcoh_2_1(n3, 0), dEcoh_1_2(n3, 0), dEcoh_1_1(n3, 0);
    std::vector<double> dV_22_2(n3, 0), dV_11_1(n3, 0), dV_21_2(n3, 0), dV_21_1(n3, 0), dV_12_1(n3, 0),
        dV_12_2(n3, 0);
    std::vector<double> dvref_2_2(n3, 0), dvref_2_1(n3, 0), dvref_1_2(n3, 0), dvref_1_1(n3, 0);
    std::vector<double> dsigma_22(n4, 0), dsigma_21_1(n4, 0), dsigma_11(n4, 0), dsigma_12_2(n4, 0);
    std::vector<double> ds_2_2(n4, 0), ds_1_1(n4, 0), ds_2_1(n4, 0), ds_1_2(n4, 0);

    const double eta2_1 = par(u, type1, P_ETA2), eta2_2 = par(u, type2, P_ETA2);
    for (int i = 0; i < N - 1; ++i) {
        const int idx_i = u->idx[i];
        for (int j = i + 1; j < N; ++j) {
            const int idx_j = u->idx[j];
            if (pes_of(u, idx_i, idx_j) != kPesEmt) continue;
            for (int b = 0; b < nb; ++b) {
                const double rijmag = distances[((size_t)j * N + i) * nb + b];
                const double *rij = &vectors[I4(0, b, i, j, nb, N)];
                if (rijmag > cutoff * rcut) continue;
                double rtemp = std::exp(acut * (rijmag - rcut));
                const double theta = 1.0 / (1 + rtemp);
                const double rtemp1 = acut * rtemp * theta;
                if (idx_i == type2 && idx_j == type2) {
                    rtemp = theta * std::exp(-eta2_2 * (rijmag - betas0_2));
                    sigma_22[I2(b, i, nb)] += rtemp;
                    sigma_22[I2(b, j, nb)] += rtemp;
                    for (int d = 0; d < 3; ++d) {
                        const double dt = (eta2_2 + rtemp1) * rtemp * rij[d] / rijmag;
                        dsigma_22[I4(d, b, i, i, nb, N)] -= dt;
                        dsigma_22[I4(d, b, j, j, nb, N)] += dt;
                        dsigma_22[I4(d, b, j, i, nb, N)] = dt;
                        dsigma_22[I4(d, b, i, j, nb, N)] = -dt;
                    }
                    rtemp = theta * std::exp(-kappadbeta_2 * (rijmag - betas0_2));
                    V_22[b] += rtemp;
                    for (int d = 0; d < 3; ++d) {
                        const double dt = (kappadbeta_2 + rtemp1) * rtemp * rij[d] / rijmag;
                        dV_22_2[I3(d, b, i, nb)] += dt;
                        dV_22_2[I3(d, b, j, nb)] -= dt;
                    }
                } else if (idx_i == type1 && idx_j == type1) {
                    rtemp = theta * std::exp(-eta2_1 * (rijmag - betas0_1));
                    sigma_11[I2(b, i, nb)] += rtemp;
                    sigma_11[I2(b, j, nb)] += rtemp;
                    for (int d = 0; d < 3; ++d) {
                        // QUIRK (pes_emt_mod.f90:705): eta2 of type2 in the type1-type1 derivative
                        const double dt = (eta2_2 + rtemp1) * rtemp * rij[d] / rijmag;
                        dsigma_11[I4(d, b, i, i, nb, N)] -= dt;
                        dsigma_11[I4(d, b, j, j, nb, N)] += dt;
                        dsigma_11[I4(d, b, j, i, nb, N)] = dt;
                        dsigma_11[I4(d, b, i, j, nb, N)] = -dt;
                    }
                    rtemp = theta * std::exp(-kappadbeta_1 * (rijmag - betas0_1));
                    V_11[b] += rtemp;
                    for (int d = 0; d < 3; ++d) {
                        const double dt = (kappadbeta_1 + rtemp1) * rtemp * rij[d] / rijmag;
                        dV_11_1[I3(d, b, i, nb)] += dt;
                        dV_11_1[I3(d, b, j, nb)] -= dt;
                    }
                } else if (idx_i != idx_j) {
                    // QUIRK (pes_emt_mod.f90:721-757): i is taken to be type1, j type2.
                    rtemp = theta * std::exp(-eta2_1 * (rijmag - betas0_1));
                    sigma_21[I2(b, j, nb)] += rtemp;
                    for (int d = 0; d < 3; ++d) {
                        const double dt = (eta2_1 + rtemp1) * rtemp * rij[d] / rijmag;
                        dsigma_21_2[I3(d, b, j, nb)] += dt;
                        dsigma_21_1[I4(d, b, i, j, nb, N)] = -dt;
                    }
                    rtemp = theta * std::exp(-eta2_2 * (rijmag - betas0_2));
                    sigma_12[I2(b, i, nb)] += rtemp;
                    for (int d = 0; d < 3; ++d) {
                        const double dt = (eta2_2 + rtemp1) * rtemp * rij[d] / rijmag;
                        dsigma_12_1[I3(d, b, i, nb)] -= dt;
                        dsigma_12_2[I4(d, b, j, i, nb, N)] = dt;
                    }
                    rtemp = theta * std::exp(-kappadbeta_1 * (rijmag - betas0_1));
                    V_21[b] += rtemp;
                    for (int d = 0; d < 3; ++d) {
                        const double dt = (kappadbeta_1 + rtemp1) * rtemp * rij[d] / rijmag;
                        dV_21_1[I3(d, b, i, nb)] += dt;
                        dV_21_2[I3(d, b, j, nb)] -= dt;
                    }
                    rtemp = theta * std::exp(-kappadbeta_2 * (rijmag - betas0_2));
                    V_12[b] += rtemp;
                    for (int d = 0; d < 3; ++d) {
                        const double dt = (kappadbeta_2 + rtemp1) * rtemp * rij[d] / rijmag;
                        dV_12_1[I3(d, b, i, nb)] += dt;
                        dV_12_2[I3(d, b, j, nb)] -= dt;
                    }
                }
            }
        }
    }

    const double v0_1 = par(u, type1, P_V0), v0_2 = par(u, type2, P_V0);
    for (auto &q : sigma_22) q *= igamma1_2;
    for (auto &q : V_22) q = q * igamma2_2 * v0_2;
    for (auto &q : sigma_11) q *= igamma1_1;
    for (auto &q : V_11) q = q * igamma2_1 * v0_1;
    for (auto &q : sigma_21) q *= igamma1_2;
    for (auto &q : sigma_12) q *= igamma1_1;
    for (auto &q : V_21) q = q * igamma2_2 * v0_2 * chi_21;
    for (auto &q : V_12) q = q * igamma2_1 * v0_1 * chi_12;
    for (auto &q : dsigma_22) q *= igamma1_2;
    for (auto &q : dsigma_11) q *= igamma1_1;
    for (auto &q : dsigma_21_2) q *= igamma1_2;
    for (auto &q : dsigma_21_1) q *= igamma1_2;
    for (auto &q : dsigma_12_1) q *= igamma1_1;
    for (auto &q : dsigma_12_2) q *= igamma1_1;
    for (auto &q : dV_22_2) q = q * igamma2_2 * v0_2;
    for (auto &q : dV_11_1) q = q * igamma2_1 * v0_1;
    for (auto &q : dV_21_2) q = q * igamma2_2 * v0_2 * chi_21;
    for (auto &q : dV_21_1) q = q * igamma2_2 * v0_2 * chi_21;
    for (auto &q : dV_12_2) q = q * igamma2_1 * v0_1 * chi_12;
    for (auto &q : dV_12_1) q = q * igamma2_1 * v0_1 * chi_12;

    for (size_t k = 0; k < n2; ++k) s_1[k] = std::max(kF1em30, sigma_11[k] + chi_12 * sigma_12[k]);
    for (size_t k = 0; k < n2; ++k) s_2[k] = std::max(kF1em30, sigma_22[k] + chi_21 * sigma_21[k]);
    for (size_t k = 0; k < n4; ++k) ds_1_1[k] = -dsigma_11[k];
    for (size_t k = 0; k < n4; ++k) ds_2_2[k] = -dsigma_22[k];

    for (int i = 0; i < N; ++i) {
        if (u->idx[i] == type2) {
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d)
                    ds_2_2[I4(d, b, i, i, nb, N)] = ds_2_2[I4(d, b, i, i, nb, N)] -
                                                    chi_21 * dsigma_21_2[I3(d, b, i, nb)];
            for (int j = 0; j < N; ++j) {
                if (u->idx[j] == type2) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            ds_2_2[I4(d, b, i, j, nb, N)] =
                                ds_2_2[I4(d, b, i, j, nb, N)] / (betaeta2_2 * s_2[I2(b, j, nb)]);
                } else if (u->idx[j] == type1) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            ds_1_2[I4(d, b, i, j, nb, N)] =
                                -chi_12 * dsigma_12_2[I4(d, b, i, j, nb, N)] / (betaeta2_1 * s_1[I2(b, j, nb)]);
                }
            }
        } else if (u->idx[i] == type1) {
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d)
                    ds_1_1[I4(d, b, i, i, nb, N)] = ds_1_1[I4(d, b, i, i, nb, N)] -
                                                    chi_12 * dsigma_12_1[I3(d, b, i, nb)];
            for (int j = 0; j < N; ++j) {
                if (u->idx[j] == type1) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            ds_1_1[I4(d, b, i, j, nb, N)] =
                                ds_1_1[I4(d, b, i, j, nb, N)] / (betaeta2_1 * s_1[I2(b, j, nb)]);
                } else if (u->idx[j] == type2) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            ds_2_1[I4(d, b, i, j, nb, N)] =
                                -chi_21 * dsigma_21_1[I4(d, b, i, j, nb, N)] / (betaeta2_2 * s_2[I2(b, j, nb)]);
                }
            }
        }
    }
    for (auto &q : s_1) q = -std::log(std::max(kTolerance, q) * kTwelfth) / betaeta2_1;
    for (auto &q : s_2) q = -std::log(std::max(kTolerance, q) * kTwelfth) / betaeta2_2;

    const double rtemp1 = 0.5 / kBohr2Ang - betaeta2_1;
    const double rtemp2 = 0.5 / kBohr2Ang - betaeta2_2;
    const double lam1 = par(u, type1, P_LAMBDA), lam2 = par(u, type2, P_LAMBDA);
    for (int i = 0; i < N; ++i) {
        for (int b = 0; b < nb; ++b) {
            const size_t k = I2(b, i, nb);
            if (u->idx[i] == type1) {
                u->dens[k] = par(u, type1, P_N0) * std::exp(rtemp1 * s_1[k]);
                exp_lambda_s1[k] = std::exp(-lam1 * s_1[k]);
                Ecoh_1[b] += ((1 + lam1 * s_1[k]) * exp_lambda_s1[k] - 1);
            } else if (u->idx[i] == type2) {
                u->dens[k] = par(u, type2, P_N0) * std::exp(rtemp2 * s_2[k]);
                exp_lambda_s2[k] = std::exp(-lam2 * s_2[k]);
                Ecoh_2[b] += ((1 + lam2 * s_2[k]) * exp_lambda_s2[k] - 1);
            }
        }
    }
    for (auto &q : Ecoh_1) q *= par(u, type1, P_E0);
    for (auto &q : Ecoh_2) q *= par(u, type2, P_E0);

    for (int i = 0; i < N; ++i) {
        if (u->idx[i] == type2) {
            for (int j = 0; j < N; ++j) {
                if (u->idx[j] == type2) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dEcoh_2_2[I3(d, b, i, nb)] += s_2[I2(b, j, nb)] * exp_lambda_s2[I2(b, j, nb)] *
                                                         ds_2_2[I4(d, b, i, j, nb, N)];
                } else if (u->idx[j] == type1) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dEcoh_1_2[I3(d, b, i, nb)] += s_1[I2(b, j, nb)] * exp_lambda_s1[I2(b, j, nb)] *
                                                         ds_1_2[I4(d, b, i, j, nb, N)];
                }
            }
        } else if (u->idx[i] == type1) {
            for (int j = 0; j < N; ++j) {
                if (u->idx[j] == type2) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dEcoh_2_1[I3(d, b, i, nb)] += s_2[I2(b, j, nb)] * exp_lambda_s2[I2(b, j, nb)] *
                                                         ds_2_1[I4(d, b, i, j, nb, N)];
                } else if (u->idx[j] == type1) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dEcoh_1_1[I3(d, b, i, nb)] += s_1[I2(b, j, nb)] * exp_lambda_s1[I2(b, j, nb)] *
                                                         ds_1_1[I4(d, b, i, j, nb, N)];
                }
            }
        }
    }
    {
        const double c2 = par(u, type2, P_E0) * lam2 * lam2, c1 = par(u, type1, P_E0) * lam1 * lam1;
        for (auto &q : dEcoh_2_2) q = c2 * q;
        for (auto &q : dEcoh_1_2) q = c1 * q;
        for (auto &q : dEcoh_2_1) q = c2 * q;
        for (auto &q : dEcoh_1_1) q = c1 * q;
    }

    const double kap1 = par(u, type1, P_KAPPA), kap2 = par(u, type2, P_KAPPA);
    for (int i = 0; i < N; ++i) {
        if (u->idx[i] == type2) {
            for (int b = 0; b < nb; ++b) {
                rtemp_beads[b] = std::exp(-kap2 * s_2[I2(b, i, nb)]);
                vref_2[b] += rtemp_beads[b];
            }
            for (int j = 0; j < N; ++j) {
                if (u->idx[j] == type2) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dvref_2_2[I3(d, b, j, nb)] += rtemp_beads[b] * ds_2_2[I4(d, b, j, i, nb, N)];
                } else if (u->idx[j] == type1) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dvref_2_1[I3(d, b, j, nb)] += rtemp_beads[b] * ds_2_1[I4(d, b, j, i, nb, N)];
                }
            }
        } else if (u->idx[i] == type1) {
            for (int b = 0; b < nb; ++b) {
                rtemp_beads[b] = std::exp(-kap1 * s_1[I2(b, i, nb)]);
                vref_1[b] += rtemp_beads[b];
            }
            for (int j = 0; j < N; ++j) {
                if (u->idx[j] == type1) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dvref_1_1[I3(d, b, j, nb)] += rtemp_beads[b] * ds_1_1[I4(d, b, j, i, nb, N)];
                } else if (u->idx[j] == type2) {
                    for (int b = 0; b < nb; ++b)
                        for (int d = 0; d < 3; ++d)
                            dvref_1_2[I3(d, b, j, nb)] += rtemp_beads[b] * ds_1_2[I4(d, b, j, i, nb, N)];
                }
            }
        }
    }
    {
        double rtemp = 12 * v0_2;
        for (auto &q : vref_2) q *= rtemp;
        for (auto &q : dvref_2_2) q = q * rtemp * kap2;
        for (auto &q : dvref_2_1) q = q * rtemp * kap2;
        rtemp = 12 * v0_1;
        for (auto &q : vref_1) q *= rtemp;
        for (auto &q : dvref_1_2) q = q * rtemp * kap1;
        for (auto &q : dvref_1_1) q = q * rtemp * kap1;
    }
    for (int b = 0; b < nb; ++b)
        u->epot[b] = u->epot[b] + (Ecoh_2[b] + Ecoh_1[b] - V_22[b] - V_11[b] -
                                   0.5 * (V_21[b] + V_12[b] - vref_2[b] - vref_1[b]));
    for (int i = 0; i < N; ++i) {
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < 3; ++d) {
                const size_t k = I3(d, b, i, nb);
                if (u->idx[i] == type2)
                    u->f[k] = u->f[k] + (dEcoh_2_2[k] + dEcoh_1_2[k] - dV_22_2[k] -
                                         0.5 * (dV_21_2[k] + dV_12_2[k] - dvref_2_2[k] - dvref_1_2[k]));
                else if (u->idx[i] == type1)
                    u->f[k] = u->f[k] + (dEcoh_2_1[k] + dEcoh_1_1[k] - dV_11_1[k] -
                                         0.5 * (dV_21_1[k] + dV_12_1[k] - dvref_2_1[k] - dvref_1_1[k]));
            }
    }
}

// build_cjk, rpmd.f90:36-59 (j is 1-based in the cosine/sine arguments)
std::vector<double> build_cjk(int nb) {
    std::vector<double> c((size_t)nb * nb);
    for (int j = 1; j <= nb; ++j)
        for (int k = 0; k <= nb - 1; ++k) {
            double v;
            if (k == 0) v = std::sqrt(1.0 / nb);
            else if (1 <= k && k <= nb / 2 - 1) v = std::sqrt(2.0 / nb) * std::cos(2.0 * kPi * j * k / nb);
            else if (k == nb / 2) v = std::sqrt(1.0 / nb) * ((j % 2) ? -1.0 : 1.0);
            else v = std::sqrt(2.0 / nb) * std::sin(2.0 * kPi * j * k / nb);
            c[(size_t)k * nb + (j - 1)] = v;  // cjk(j,k+1), column major
        }
    return c;
}
inline double cjk_at(const std::vector<double> &c, int nb, int j0, int k0) { return c[(size_t)k0 * nb + j0]; }

double temp_of(const orc_universe *u, const orc_params *p, int i) {
    return u->is_proj[u->idx[i] - 1] ? p->Tproj : p->Tsurf;
}
int algo_of(const orc_universe *u, int i) { return u->algo[u->idx[i] - 1]; }

bool any_algo(const orc_universe *u, int id) {
    for (int t = 0; t < u->ntypes; ++t)
        if (u->algo[t] == id) return true;
    return false;
}

// verlet_1 / verlet_2, md_algo.f90:110-142
void verlet_1(orc_universe *u, const orc_params *p, int i) {
    const int nb = u->nbeads;
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d) {
            const size_t k = I3(d, b, i, nb);
            if (!u->is_fixed[k]) u->v[k] = u->v[k] + 0.5 * p->step * u->a[k];
            else u->v[k] = 0.0;
        }
    if (nb == 1)
        for (int d = 0; d < 3; ++d) {
            const size_t k = I3(d, 0, i, nb);
            if (!u->is_fixed[k]) u->r[k] = u->r[k] + p->step * u->v[k];
        }
}
void verlet_2(orc_universe *u, const orc_params *p, int i) {
    const int nb = u->nbeads;
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d) {
            const size_t k = I3(d, b, i, nb);
            if (!u->is_fixed[k]) u->v[k] = u->v[k] + 0.5 * p->step * u->a[k];
            else u->v[k] = 0.0;
        }
}

// Langevin coefficients shared by langevin_1/2, md_algo.f90:165-198 and 253-285.
struct LangCoef { double c0, c1, c2, sigma_r, sigma_v, c_rv; };
void langevin_coefs(const orc_universe *u, const orc_params *p, int i, const double *xi,
                    std::vector<LangCoef> &out, bool second) {
    const int nb = u->nbeads;
    const double temp = kB * nb * temp_of(u, p, i) / u->m[i];
    out.resize(nb);
    bool all_big = true;
    for (int b = 0; b < nb; ++b)
        if (!(xi[b] * p->step > kF1em2)) all_big = false;
    for (int b = 0; b < nb; ++b) {
        const double xidt = xi[b] * p->step, xidt2 = xidt * xidt, ixidt = p->step / xidt;
        LangCoef &c = out[b];
        if (all_big && temp > kTolerance) {
            c.c0 = std::exp(-xidt);
            c.c1 = (1 - c.c0) * ixidt;
            c.c2 = (1 - c.c1 / p->step) * ixidt;
            c.sigma_r = ixidt * std::sqrt(temp * (2 * xidt - 3 + 4 * c.c0 - c.c0 * c.c0));
            c.sigma_v = std::sqrt(temp * (1 - c.c0 * c.c0));
            c.c_rv = ixidt * temp * (1 - c.c0) * (1 - c.c0) / (c.sigma_r * c.sigma_v);
        } else {
            c.c0 = 1 - xidt + 0.5 * xidt2;
            c.c1 = (1 - 0.5 * xidt + 2 * kTwelfth * xidt2) * p->step;
            c.c2 = (0.5 - 2 * kTwelfth * xidt + 0.5 * kTwelfth * xidt2) * p->step;
            c.sigma_r = second ? 0.0 : p->step * std::sqrt(temp * (8 * kTwelfth * xidt - 0.5 * xidt2));
            c.sigma_v = std::sqrt(2 * temp * xidt * (1 - xidt));
            c.c_rv = 0.5 * kSqrt3 * (1 - 0.125 * xidt);
        }
    }
}

// friction source: LDFA-converted EMT density (algo 1003) or a constant (1007)
void friction_of(const orc_universe *u, const orc_params *p, int i, std::vector<double> &xi) {
    const int nb = u->nbeads;
    xi.resize(nb);
    for (int b = 0; b < nb; ++b)
        xi[b] = (algo_of(u, i) == ORC_LANGEVIN_CONST) ? p->gamma_const : u->dens[I2(b, i, nb)];
}

// langevin_1, md_algo.f90:146-232
void langevin_1(orc_universe *u, const orc_params *p, int i, const double *randy) {
    const int nb = u->nbeads;
    std::vector<double> xi;
    friction_of(u, p, i, xi);
    std::vector<LangCoef> c;
    langevin_coefs(u, p, i, xi.data(), c, false);
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d) {
            const size_t k = I3(d, b, i, nb);
            if (!u->is_fixed[k]) {
                u->r[k] = u->r[k] + c[b].c1 * u->v[k] + c[b].c2 * p->step * u->a[k] + c[b].sigma_r * randy[k];
                u->v[k] = c[b].c0 * u->v[k] + (c[b].c1 - c[b].c2) * u->a[k] + c[b].sigma_v * c[b].c_rv * randy[k];
            } else {
                u->v[k] = 0.0;
            }
        }
}

// langevin_2, md_algo.f90:236-300
void langevin_2(orc_universe *u, const orc_params *p, int i, const double *randy) {
    const int nb = u->nbeads;
    std::vector<double> xi;
    friction_of(u, p, i, xi);
    std::vector<LangCoef> c;
    langevin_coefs(u, p, i, xi.data(), c, true);
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d) {
            const size_t k = I3(d, b, i, nb);
            if (!u->is_fixed[k])
                u->v[k] = u->v[k] + c[b].c2 * u->a[k] + c[b].sigma_v * std::sqrt(1 - c[b].c_rv * c[b].c_rv) * randy[k];
            else
                u->v[k] = 0.0;
        }
}

// ldfa, md_algo.f90:506-570 (converts dens(:,i) to a friction coefficient in place)
int ldfa(orc_universe *u, int i) {
    const int nb = u->nbeads;
    const double convert = 1.00794 * kAmu2Mass;
    const double coefs[12] = {0.0802484, -1.12851, 9.28508, 2.10064, -843.419, 8.85354e3, -4.89023e4,
                              1.6741e5, -3.67098e5, 5.03476e5, -3.9426e5, 1.34763e5};
    for (int b = 0; b < nb; ++b) {
        const size_t k = I2(b, i, nb);
        double fric = u->dens[k];
        if (kFm1em12 <= fric && fric <= kF036) {
            fric = 0.0;
            double temp = u->dens[k];
            for (int j = 0; j < 12; ++j) {
                fric = fric + coefs[j] * temp;
                temp = temp * u->dens[k];
            }
        } else if (fric > kF036) {
            fric = 0.001 * (4.7131 - std::exp(-4.41305 * fric));
        } else {
            return -3;  // "EMT density array contains negative values."
        }
        u->dens[k] = fric;
    }
    for (int b = 0; b < nb; ++b) {
        const size_t k = I2(b, i, nb);
        u->dens[k] = u->dens[k] * convert / kHbar / u->m[i];
    }
    return 0;
}

// andersen, md_algo.f90:402-432 (deviates injected)
void andersen(orc_universe *u, const orc_params *p, int i, const double *nv, const double *uu) {
    const int nb = u->nbeads;
    const double ibetaN = nb * kB * temp_of(u, p, i);
    const double sd = std::sqrt(ibetaN / u->m[i]);
    const double thr = p->step / p->andersen_time;
    for (int b = 0; b < nb; ++b)
        if (uu[I2(b, i, nb)] < thr)
            for (int d = 0; d < 3; ++d) {
                const size_t k = I3(d, b, i, nb);
                if (!u->is_fixed[k]) u->v[k] = nv[k] * sd + 0.0;
            }
}

// pile_thermostat, md_algo.f90:440-502 (zeta injected)
void pile(orc_universe *u, const orc_params *p, int i, const std::vector<double> &cjk, const double *zeta) {
    const int nb = u->nbeads;
    const double betaN = 1.0 / (kB * temp_of(u, p, i) * nb);
    std::vector<double> newP(3 * nb, 0.0), atomP(3 * nb), gammak(nb), c1(nb), c2(nb);
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d) atomP[b * 3 + d] = u->m[i] * u->v[I3(d, b, i, nb)];
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < nb; ++k)
            for (int d = 0; d < 3; ++d) newP[b * 3 + d] = newP[b * 3 + d] + atomP[k * 3 + d] * cjk_at(cjk, nb, k, b);
    for (int k = 0; k < nb; ++k) {
        if (k == 0) gammak[k] = 1 / p->pile_tau;
        else {
            const double wn = 1 / betaN / kHbar;
            const double wk = 2 * wn * std::sin(k * kPi / nb);
            gammak[k] = 2 * wk;
        }
    }
    for (int k = 0; k < nb; ++k) {
        c1[k] = std::exp(-0.5 * p->step * gammak[k]);
        c2[k] = std::sqrt(1 - c1[k] * c1[k]);
    }
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d)
            newP[b * 3 + d] = c1[b] * newP[b * 3 + d] + std::sqrt(u->m[i] / betaN) * c2[b] * zeta[I3(d, b, i, nb)];
    std::fill(atomP.begin(), atomP.end(), 0.0);
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < nb; ++k)
            for (int d = 0; d < 3; ++d)
                if (!u->is_fixed[I3(d, b, i, nb)])
                    atomP[b * 3 + d] = atomP[b * 3 + d] + newP[k * 3 + d] * cjk_at(cjk, nb, b, k);
    for (int b = 0; b < nb; ++b)
        for (int d = 0; d < 3; ++d) u->v[I3(d, b, i, nb)] = atomP[b * 3 + d] / u->m[i];
}

}  // namespace

extern "C" {

void orc_minimg_beads(const orc_universe *u, int i, int j, double *r, double *vec) {
    const int nb = u->nbeads;
    const double *S = u->simbox, *IS = u->isimbox;  // column major
    for (int b = 0; b < nb; ++b) {
        double v[3], w[3];
        for (int d = 0; d < 3; ++d) v[d] = u->r[I3(d, b, j, nb)] - u->r[I3(d, b, i, nb)];
        for (int d = 0; d < 3; ++d) w[d] = IS[d] * v[0] + IS[3 + d] * v[1] + IS[6 + d] * v[2];
        for (int d = 0; d < 3; ++d) w[d] = w[d] - anint(w[d]);
        for (int d = 0; d < 3; ++d) v[d] = S[d] * w[0] + S[3 + d] * w[1] + S[6 + d] * w[2];
        for (int d = 0; d < 3; ++d) vec[b * 3 + d] = v[d];
        r[b] = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
}

int orc_compute_emt(orc_universe *u, const double *distances, const double *vectors) {
    int nEMT = 0;
    for (int i = 1; i <= u->ntypes; ++i)
        if (pes_of(u, i, i) == kPesEmt) ++nEMT;
    if (nEMT == 1) emt_1species(u, distances, vectors);
    else if (nEMT == 2) emt_2species(u, distances, vectors);
    else return -2;
    return 0;
}

int orc_ring_polymer_step(orc_universe *u, const orc_params *p) {
    const int N = u->natoms, nb = u->nbeads;
    const size_t n3 = 3 * (size_t)nb * N;
    std::vector<double> cjk = build_cjk(nb);
    std::vector<double> saveR(u->r, u->r + n3), saveV(u->v, u->v + n3);
    const double prefactor = -1 * u->m[0] * std::pow(kB * p->Tproj * nb / kHbar, 2);
    std::vector<double> P(n3), Q(n3), newP(n3, 0.0), newQ(n3, 0.0);
    for (int i = 0; i < N; ++i)
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < 3; ++d) P[I3(d, b, i, nb)] = u->m[i] * u->v[I3(d, b, i, nb)];
    for (size_t k = 0; k < n3; ++k) Q[k] = u->r[k];
    for (int b = 0; b < nb; ++b)
        for (int k = 0; k < nb; ++k)
            for (int i = 0; i < N; ++i)
                for (int d = 0; d < 3; ++d) {
                    newP[I3(d, b, i, nb)] = newP[I3(d, b, i, nb)] + P[I3(d, k, i, nb)] * cjk_at(cjk, nb, k, b);
                    newQ[I3(d, b, i, nb)] = newQ[I3(d, b, i, nb)] + Q[I3(d, k, i, nb)] * cjk_at(cjk, nb, k, b);
                }
    P = newP;
    Q = newQ;
    const double piN = kPi / nb;
    std::vector<double> poly(4 * (size_t)nb);
    for (int i = 0; i < N; ++i) {
        const double mass = u->m[i];
        poly[0] = 1.0; poly[1] = 0.0; poly[2] = p->step / mass; poly[3] = 1.0;
        const double betaN = 1.0 / (kB * temp_of(u, p, i) * nb);
        if (nb > 1) {
            const double twown = 2.0 / betaN / kHbar;
            for (int b = 1; b <= nb / 2; ++b) {
                const double wk = twown * std::sin(b * piN), wt = wk * p->step, wm = wk * mass;
                const double cw = std::cos(wt), sw = std::sin(wt);
                poly[4 * b + 0] = cw;
                poly[4 * b + 1] = -wm * sw;
                poly[4 * b + 2] = sw / wm;
                poly[4 * b + 3] = cw;
            }
            for (int b = 1; b <= (nb - 1) / 2; ++b)
                for (int q = 0; q < 4; ++q) poly[4 * (nb - b) + q] = poly[4 * b + q];
        }
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < 3; ++d) {
                const size_t k = I3(d, b, i, nb);
                const double p_new = P[k] * poly[4 * b + 0] + Q[k] * poly[4 * b + 1];
                Q[k] = P[k] * poly[4 * b + 2] + Q[k] * poly[4 * b + 3];
                P[k] = p_new;
            }
    }
    for (size_t k = 0; k < n3; ++k)
        if (!u->is_fixed[k]) { u->r[k] = 0.0; u->v[k] = 0.0; }
    for (int i = 0; i < N; ++i)
        for (int b = 0; b < nb; ++b)
            for (int k = 0; k < nb; ++k)
                for (int d = 0; d < 3; ++d) {
                    const size_t t = I3(d, b, i, nb);
                    if (!u->is_fixed[t]) {
                        u->r[t] = u->r[t] + Q[I3(d, k, i, nb)] * cjk_at(cjk, nb, b, k);
                        u->v[t] = u->v[t] + P[I3(d, k, i, nb)] * cjk_at(cjk, nb, b, k) / u->m[i];
                    }
                }
    if (any_algo(u, ORC_LANGEVIN) || any_algo(u, ORC_LANGEVIN_CONST)) {
        for (int i = 0; i < N; ++i) {
            const int al = algo_of(u, i);
            if (al != ORC_LANGEVIN && al != ORC_LANGEVIN_CONST) continue;
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d) {
                    u->r[I3(d, b, i, nb)] = saveR[I3(d, b, i, nb)];
                    u->v[I3(d, b, i, nb)] = saveV[I3(d, b, i, nb)];
                }
            for (int b = 0; b < nb; ++b) {
                const int prev = (b == 0) ? nb - 1 : b - 1, next = (b == nb - 1) ? 0 : b + 1;
                for (int d = 0; d < 3; ++d)
                    u->f[I3(d, b, i, nb)] = prefactor * (2 * u->r[I3(d, b, i, nb)] - u->r[I3(d, prev, i, nb)] -
                                                         u->r[I3(d, next, i, nb)]);
            }
        }
    }
    return 0;
}

int orc_calc_force(orc_universe *u, const orc_params *p) {
    const int N = u->natoms, nb = u->nbeads;
    const size_t n3 = 3 * (size_t)nb * N;
    for (size_t k = 0; k < n3; ++k) { u->f[k] = 0.0; u->a[k] = 0.0; }
    for (int b = 0; b < nb; ++b) u->epot[b] = 0.0;
    if (nb > 1) orc_ring_polymer_step(u, p);
    std::vector<double> distances((size_t)nb * N * N, 0.0), vectors(3 * (size_t)nb * N * N, 0.0);
    std::vector<double> td(nb), tv(3 * nb);
    for (int j = 0; j < N - 1; ++j)
        for (int i = j + 1; i < N; ++i) {
            orc_minimg_beads(u, i, j, td.data(), tv.data());
            for (int b = 0; b < nb; ++b) {
                distances[((size_t)j * N + i) * nb + b] = td[b];
                distances[((size_t)i * N + j) * nb + b] = td[b];
                for (int d = 0; d < 3; ++d) {
                    vectors[I4(d, b, i, j, nb, N)] = -tv[b * 3 + d];
                    vectors[I4(d, b, j, i, nb, N)] = +tv[b * 3 + d];
                }
            }
        }
    int rc = orc_compute_emt(u, distances.data(), vectors.data());
    if (rc) return rc;
    for (int i = 0; i < N; ++i)
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < 3; ++d) {
                const size_t k = I3(d, b, i, nb);
                if (!u->is_fixed[k]) u->a[k] = u->f[k] / u->m[i];
            }
    return 0;
}

void orc_remove_com_velocity(orc_universe *u) {
    const int N = u->natoms, nb = u->nbeads;
    for (int dummy = 0; dummy < 1000; ++dummy) {
        double num[3] = {0, 0, 0}, msum = 0;
        for (int i = 0; i < N; ++i)
            for (int d = 0; d < 3; ++d) {
                double s = 0;
                for (int b = 0; b < nb; ++b) s += u->v[I3(d, b, i, nb)];
                num[d] = num[d] + s * u->m[i];
            }
        for (int i = 0; i < N; ++i) msum += u->m[i];
        double vcm[3];
        for (int d = 0; d < 3; ++d) vcm[d] = num[d] / msum / nb / N;
        for (int i = 0; i < N; ++i)
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d) u->v[I3(d, b, i, nb)] = u->v[I3(d, b, i, nb)] - vcm[d];
    }
}

int orc_propagate_1(orc_universe *u, const orc_params *p, const double *randy, const double *zeta,
                    const double *andersen_v, const double *andersen_u) {
    std::vector<double> cjk;
    if (any_algo(u, ORC_PILE)) cjk = build_cjk(u->nbeads);
    for (int i = 0; i < u->natoms; ++i) {
        switch (algo_of(u, i)) {
            case ORC_VERLET: verlet_1(u, p, i); break;
            case ORC_ANDERSEN:
                verlet_1(u, p, i);
                andersen(u, p, i, andersen_v, andersen_u);
                break;
            case ORC_PILE:
                pile(u, p, i, cjk, zeta);
                verlet_1(u, p, i);
                break;
            case ORC_LANGEVIN:
            case ORC_LANGEVIN_CONST: langevin_1(u, p, i, randy); break;
            default: return -4;
        }
    }
    if (any_algo(u, ORC_ANDERSEN) || any_algo(u, ORC_PILE)) orc_remove_com_velocity(u);
    return 0;
}

int orc_propagate_2(orc_universe *u, const orc_params *p, const double *randy) {
    for (int i = 0; i < u->natoms; ++i) {
        switch (algo_of(u, i)) {
            case ORC_VERLET:
            case ORC_ANDERSEN:
            case ORC_PILE: verlet_2(u, p, i); break;
            case ORC_LANGEVIN: {
                int rc = ldfa(u, i);
                if (rc) return rc;
                langevin_2(u, p, i, randy);
                break;
            }
            case ORC_LANGEVIN_CONST: langevin_2(u, p, i, randy); break;
            default: return -4;
        }
    }
    return 0;
}

void orc_atom_ekin(const orc_universe *u, double *ekin_p, double *ekin_l) {
    const int nb = u->nbeads;
    double ep = 0, el = 0;
    for (int i = 0; i < u->natoms; ++i) {
        double s2 = 0;
        for (int d = 0; d < 3; ++d) {
            double s = 0;
            for (int b = 0; b < nb; ++b) s += u->v[I3(d, b, i, nb)];
            s2 += s * s;
        }
        const double nrg = u->m[i] * s2;
        if (u->is_proj[u->idx[i] - 1]) ep += nrg; else el += nrg;
    }
    *ekin_p = 0.5 * ep / nb / nb;
    *ekin_l = 0.5 * el / nb / nb;
}

void orc_bead_ekin(const orc_universe *u, double *ekin_p, double *ekin_l) {
    const int nb = u->nbeads;
    double ep = 0, el = 0;
    for (int i = 0; i < u->natoms; ++i) {
        double s2 = 0;
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < 3; ++d) s2 += u->v[I3(d, b, i, nb)] * u->v[I3(d, b, i, nb)];
        const double nrg = u->m[i] * s2;
        if (u->is_proj[u->idx[i] - 1]) ep += nrg; else el += nrg;
    }
    *ekin_p = 0.5 * ep / nb;
    *ekin_l = 0.5 * el / nb;
}

double orc_bead_epot(const orc_universe *u, const orc_params *p) {
    const int nb = u->nbeads;
    if (nb == 1) return 0.0;
    double epot = 0.0;
    for (int i = 0; i < u->natoms; ++i) {
        const double T = u->is_proj[u->idx[i] - 1] ? p->Tproj : p->Tsurf;
        const double wn2 = std::pow(kB * T * nb / kHbar, 2);
        double s = 0;
        for (int b = 0; b < nb; ++b) {
            const int k = (b + 1) % nb;
            double dd = 0;
            for (int d = 0; d < 3; ++d) {
                const double x = u->r[I3(d, b, i, nb)] - u->r[I3(d, k, i, nb)];
                dd += x * x;
            }
            s += dd;  // dx(b,i)**2 with dx = sqrt(dd)
        }
        epot = epot + u->m[i] * s * wn2;
    }
    return 0.5 * epot / nb;
}

int orc_md_step(orc_universe *u, const orc_params *p, const double *randy, const double *zeta,
                const double *andersen_v, const double *andersen_u) {
    int rc = orc_propagate_1(u, p, randy, zeta, andersen_v, andersen_u);
    if (rc) return rc;
    rc = orc_calc_force(u, p);
    if (rc) return rc;
    return orc_propagate_2(u, p, randy);
}

int orc_run_verlet(orc_universe *u, const orc_params *p, int nsteps, double pul) {
    const int nb = u->nbeads;
    int istep;
    for (istep = 1; istep <= nsteps; ++istep) {
        if (orc_md_step(u, p, nullptr, nullptr, nullptr, nullptr)) return -istep;
        bool all_above = true;
        for (int b = 0; b < nb; ++b)
            if (!(u->r[I3(2, b, 0, nb)] > pul)) all_above = false;
        if (all_above && u->is_proj[u->idx[0] - 1]) break;
    }
    return istep > nsteps ? nsteps : istep;
}

namespace {
// splitmix64 (Steele, Lea, Flood, OOPSLA 2014): 64-bit counter generator
struct SplitMix {
    uint64_t x;
    uint64_t next() {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double u01() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }  // (0, 1)
    double normal() { return std::sqrt(-2.0 * std::log(u01())) * std::cos(2.0 * kPi * u01()); }
};
}  // namespace

int64_t orc_run_steps(orc_universe **u, int n, const orc_params *p, double seconds, int64_t max_sweeps,
                      uint64_t seed, double *elapsed) {
    size_t mx = 0;
    for (int k = 0; k < n; ++k) mx = std::max(mx, (size_t)3 * u[k]->nbeads * u[k]->natoms);
    std::vector<double> randy(mx), zeta(mx), av(mx), au(mx);
    SplitMix g{seed};
    const auto t0 = std::chrono::steady_clock::now();
    int64_t atom_steps = 0;
    double el = 0.0;
    for (int64_t sweep = 0; sweep < max_sweeps; ++sweep) {
        for (int k = 0; k < n; ++k) {
            const size_t m = (size_t)3 * u[k]->nbeads * u[k]->natoms;
            for (size_t i = 0; i < m; ++i) {
                randy[i] = g.normal();
                zeta[i] = g.normal();
                av[i] = g.normal();
                au[i] = g.u01();
            }
            if (orc_md_step(u[k], p, randy.data(), zeta.data(), av.data(), au.data())) return -1;
            atom_steps += (int64_t)u[k]->natoms * u[k]->nbeads;
        }
        el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el >= seconds) break;
    }
    if (elapsed) *elapsed = el;
    return atom_steps;
}

}  // extern "C"
