/*
 * nene_oracle.cpp -- CPU FP64 restatement of the RuNNer short-range prediction used by
 * md_tian2's compute_nene (src/pes_nene_mod.f90:7145-7368).  TEST INFRASTRUCTURE ONLY:
 * the checker for the CUDA HDNNP/surrogate kernels; never part of the product path.
 *
 * It follows the vendored RuNNer routines loop by loop:
 *   neighbour list            RuNNer_src/neighbor_para_short.f90:59-207 (i -> j -> n1 -> n2 -> n3)
 *   neighbour index maps      RuNNer_src/getneighboridxatomic_para.f90:54-71
 *   per-atom prediction       RuNNer_src/getshortatomic.f90:113-359 (forward-mode dG/dx)
 *   radial G2                 RuNNer_src/atomsymfunction2.f90:80-170
 *   angular G3                RuNNer_src/atomsymfunction3Andi.f90:90-257
 *   cutoff functions          RuNNer_src/getcutoff.f90:51-162
 *   MLP forward / derivative  RuNNer_src/calconenn.f90:83-153, getdnodes_values.f90:65-114
 *   cell wrap                 RuNNer_src/translate.f90 (as fractional-coordinate folding)
 * Parity: unpinned by a reference run (no Fortran compiler); pinned by the shipped
 * C-graphene network (example/md/RuNNer_input) through finite differences and the
 * force-sum check of pes_nene_mod.f90:7272-7287.
 */
#include <cmath>
#include <cstdint>
#include <vector>

extern "C" {

typedef struct orc_nn {
    int nelem;
    const int *z;          /* nuclear charge per element index (ascending) */
    int maxsf;
    const int *nsf;        /* per element */
    /* per element e and symmetry function s at [e*maxsf + s] */
    const int *sftype;
    const double *eta, *rshift, *lambda, *zeta, *rc; /* bohr units */
    const int *e1, *e2;    /* neighbour element nuclear charges */
    const double *smin, *smax, *savg;
    int scalesym, centersym;
    double scmin, scmax;
    int cutoff_type;
    double cutoff_alpha;
    int nlayers;           /* hidden + output */
    int maxnodes;
    const int *nodes;      /* per element (nlayers+1) entries, nodes[0] = nsf */
    const char *act;       /* per element nlayers*maxnodes activation letters */
    int maxweights;
    const double *weights; /* per element maxweights */
    int normnodes;
    int remove_atom_energies;
    const double *atom_energy; /* Ha per element */
} orc_nn;

}  // extern "C"

namespace {

const double kPi = 3.14159265358979323846264338327950288;
const double kAng2Bohr = 1.0 / 0.529177211;
const double kHa2eV = 27.21138602;

struct Neighbor {
    double x, y, z, r;
    int j, n1, n2, n3, elem;
};

// getcutoff.f90:51-162 (types 0..8)
void getcutoff(int type, double alpha, double rc, double r, double &fc, double &dfc) {
    const double rtemp = r / rc, rci = alpha * rc, iw = 1.0 / (rc - rci);
    if (type == 0) { fc = 1.0; dfc = 0.0; return; }
    if (r <= rci && type != 2 && type != 3) { fc = 1.0; dfc = 0.0; return; }
    const double x = (r - rci) * iw;
    switch (type) {
        case 1: fc = 0.5 * (std::cos(kPi * x) + 1.0); dfc = (-std::sin(kPi * x)) * (kPi / 2.0) * iw; break;
        case 2: {
            if (r <= rci) { fc = std::pow(std::tanh(1.0), 3); dfc = 0.0; break; }
            const double t = std::tanh(1.0 - rtemp);
            fc = t * t * t;
            dfc = (-3.0 / rc) * (t * t - t * t * t * t);
            break;
        }
        case 3: {
            const double c = std::pow((std::exp(1.0) + 1.0) / (std::exp(1.0) - 1.0), 3);
            if (r <= rci) { fc = c * std::pow(std::tanh(1.0), 3); dfc = 0.0; break; }
            const double t = std::tanh(1.0 - rtemp);
            fc = c * t * t * t;
            dfc = c * ((-3.0 / rc) * (t * t - t * t * t * t));
            break;
        }
        case 4:
            fc = std::exp(1.0 - 1.0 / (1.0 - x * x));
            dfc = (-2.0 * iw * x / ((1.0 - x * x) * (1.0 - x * x))) * std::exp(-1.0 / (1.0 - x * x)) * std::exp(1.0);
            break;
        case 5: fc = (2.0 * x - 3.0) * x * x + 1.0; dfc = iw * x * (6.0 * x - 6.0); break;
        case 6: fc = ((15.0 - 6.0 * x) * x - 10.0) * x * x * x + 1.0; dfc = iw * x * x * ((60.0 - 30.0 * x) * x - 30.0); break;
        case 7:
            fc = (x * (x * (20.0 * x - 70.0) + 84.0) - 35.0) * x * x * x * x + 1.0;
            dfc = (x * x * x) * iw * (x * (x * (140.0 * x - 420.0) + 420.0) - 140.0);
            break;
        default:
            fc = (x * (x * (x * (315.0 - 70.0 * x) - 540.0) + 420.0) - 126.0) * std::pow(x, 5) + 1.0;
            dfc = iw * std::pow(x, 4) * (x * (x * ((2520.0 - 630.0 * x) * x - 3780.0) + 2520.0) - 630.0);
            break;
    }
}

double act_f(char a, double x) {
    switch (a) {
        case 't': return std::tanh(x);
        case 'g': return std::exp(-0.5 * x * x);
        case 'l': return x;
        case 'c': return std::cos(x);
        case 's': return 1.0 / (1.0 + std::exp(-1.0 * x));
        case 'S': return 1.0 - 1.0 / (1.0 + std::exp(-1.0 * x));
        case 'e': return std::exp(-1.0 * x);
        case 'p': return std::log(std::exp(x) + 1.0);
        case 'h': return x * x;
        default: return NAN;
    }
}

double act_d(char a, double sum, double val) {
    switch (a) {
        case 'l': return 1.0;
        case 't': return 1.0 - val * val;
        case 'g': return -2.0 * 0.5 * sum * val;
        case 'c': return -1.0 * std::sin(sum);
        case 's': return std::exp(-1.0 * sum) / std::pow(1.0 + std::exp(-1.0 * sum), 2.0);
        case 'S': return -1.0 * std::exp(-1.0 * sum) / std::pow(1.0 + std::exp(-1.0 * sum), 2.0);
        case 'e': return -1.0 * val;
        case 'p': return (std::exp(val) - 1.0) / std::exp(val);
        case 'h': return 2.0 * sum;
        default: return NAN;
    }
}

// neighbor_para_short.f90:59-207 (periodic branch and non-periodic branch)
void build_neighbors(int N, const double *xyz, const double *lat, bool periodic, double cutoff, const int *zat,
                     std::vector<std::vector<Neighbor>> &nb) {
    nb.assign(N, {});
    int na = 0, nbb = 0, nc = 0;
    if (periodic) {
        auto L = [&](int i, int k) { return lat[3 * (i - 1) + (k - 1)]; };  // lattice(i,k), row i = vector i
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
        const double proja = std::fabs(L(1, 1) * bxc[0] + L(1, 2) * bxc[1] + L(1, 3) * bxc[2]);
        const double projb = std::fabs(L(2, 1) * axc[0] + L(2, 2) * axc[1] + L(2, 3) * axc[2]);
        const double projc = std::fabs(L(3, 1) * axb[0] + L(3, 2) * axb[1] + L(3, 3) * axb[2]);
        while ((double)na * proja <= cutoff) ++na;
        while ((double)nbb * projb <= cutoff) ++nbb;
        while ((double)nc * projc <= cutoff) ++nc;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                for (int n1 = -na; n1 <= na; ++n1)
                    for (int n2 = -nbb; n2 <= nbb; ++n2)
                        for (int n3 = -nc; n3 <= nc; ++n3) {
                            if (n1 == 0 && n2 == 0 && n3 == 0 && i == j) continue;
                            const double xt = xyz[3 * j] + n1 * L(1, 1) + n2 * L(2, 1) + n3 * L(3, 1);
                            const double yt = xyz[3 * j + 1] + n1 * L(1, 2) + n2 * L(2, 2) + n3 * L(3, 2);
                            const double zt = xyz[3 * j + 2] + n1 * L(1, 3) + n2 * L(2, 3) + n3 * L(3, 3);
                            const double d1 = xt - xyz[3 * i], d2 = yt - xyz[3 * i + 1], d3 = zt - xyz[3 * i + 2];
                            const double rr = d1 * d1 + d2 * d2 + d3 * d3;
                            if (rr <= cutoff * cutoff)
                                nb[i].push_back(Neighbor{xt, yt, zt, std::sqrt(rr), j, n1, n2, n3, zat[j]});
                        }
    } else {
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                if (i == j) continue;
                const double d1 = xyz[3 * j] - xyz[3 * i], d2 = xyz[3 * j + 1] - xyz[3 * i + 1],
                             d3 = xyz[3 * j + 2] - xyz[3 * i + 2];
                const double rr = d1 * d1 + d2 * d2 + d3 * d3;
                if (rr <= cutoff * cutoff)
                    nb[i].push_back(Neighbor{xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], std::sqrt(rr), j, 0, 0, 0, zat[j]});
            }
    }
}

// fold positions into the cell (RuNNer_src/translate.f90 keeps every atom inside the
// parallelepiped spanned by the lattice vectors)
void wrap(int N, double *xyz, const double *lat) {
    // fractional coordinates: xyz = f1*a1 + f2*a2 + f3*a3, lat rows are a_i
    double A[9];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) A[k * 3 + i] = lat[3 * i + k];  // column i = a_i
    const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                       A[2] * (A[3] * A[7] - A[4] * A[6]);
    double I[9];
    I[0] = (A[4] * A[8] - A[5] * A[7]) / det; I[1] = (A[2] * A[7] - A[1] * A[8]) / det; I[2] = (A[1] * A[5] - A[2] * A[4]) / det;
    I[3] = (A[5] * A[6] - A[3] * A[8]) / det; I[4] = (A[0] * A[8] - A[2] * A[6]) / det; I[5] = (A[2] * A[3] - A[0] * A[5]) / det;
    I[6] = (A[3] * A[7] - A[4] * A[6]) / det; I[7] = (A[1] * A[6] - A[0] * A[7]) / det; I[8] = (A[0] * A[4] - A[1] * A[3]) / det;
    for (int a = 0; a < N; ++a) {
        double f[3];
        for (int i = 0; i < 3; ++i) f[i] = I[3 * i] * xyz[3 * a] + I[3 * i + 1] * xyz[3 * a + 1] + I[3 * i + 2] * xyz[3 * a + 2];
        for (int i = 0; i < 3; ++i) {
            const double s = std::floor(f[i]);
            if (s != 0.0)
                for (int k = 0; k < 3; ++k) xyz[3 * a + k] -= s * lat[3 * i + k];
        }
    }
}

}  // namespace

extern "C" {

/* Neighbour list in RuNNer order for the bit-exact test.  Positions in bohr (folded
   into the cell first, as in orc_nene_energy_force), lattice rows in bohr.  out_j/out_n (3 per entry) sized by the caller (max_total); returns the
   number of entries, counts[i] = neighbours of atom i; -1 if max_total is too small. */
int orc_nene_neighbors(int N, const double *xyz_bohr, const double *lat_bohr, int periodic, double cutoff,
                       int *counts, int *out_j, int *out_n, double *out_r, int max_total) {
    std::vector<int> z(N, 0);
    std::vector<double> xyz(xyz_bohr, xyz_bohr + 3 * N);
    if (periodic) wrap(N, xyz.data(), lat_bohr);  // same cell folding as compute_nene
    std::vector<std::vector<Neighbor>> nb;
    build_neighbors(N, xyz.data(), lat_bohr, periodic != 0, cutoff, z.data(), nb);
    int tot = 0;
    for (int i = 0; i < N; ++i) {
        counts[i] = (int)nb[i].size();
        for (const Neighbor &q : nb[i]) {
            if (tot >= max_total) return -1;
            out_j[tot] = q.j;
            out_n[3 * tot] = q.n1; out_n[3 * tot + 1] = q.n2; out_n[3 * tot + 2] = q.n3;
            out_r[tot] = q.r;
            ++tot;
        }
    }
    return tot;
}

/* compute_nene for one bead: positions in A (3,N), cell columns in A (simbox, column
   major), elem: 0-based element index per atom.  Outputs eV and eV/A; G (N x maxsf,
   scaled) and per-atom energies (eV) optional. */
int orc_nene_energy_force(const orc_nn *nn, int N, const int *elem, const double *r_ang, const double *simbox,
                          double *energy_ev, double *forces, double *G_out, double *eatom_out) {
    std::vector<double> xyz(3 * N);
    for (int k = 0; k < 3 * N; ++k) xyz[k] = r_ang[k] * kAng2Bohr;
    double lat[9];
    bool periodic = false;
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            lat[3 * i + k] = simbox[3 * i + k] * kAng2Bohr;  // lattice(i,:) = simbox(:,i)
            if (simbox[3 * i + k] != 0.0) periodic = true;
        }
    if (periodic) wrap(N, xyz.data(), lat);
    std::vector<int> zat(N);
    for (int a = 0; a < N; ++a) zat[a] = nn->z[elem[a]];
    double maxcut = 0.0;
    for (int e = 0; e < nn->nelem; ++e)
        for (int s = 0; s < nn->nsf[e]; ++s) maxcut = std::max(maxcut, nn->rc[e * nn->maxsf + s]);
    std::vector<std::vector<Neighbor>> nb;
    build_neighbors(N, xyz.data(), lat, periodic, maxcut, zat.data(), nb);

    std::vector<double> F(3 * N, 0.0);
    double etot = 0.0;
    for (int i1 = 0; i1 < N; ++i1) {
        const int e = elem[i1];
        const int nsf = nn->nsf[e];
        const auto &L = nb[i1];
        const int nn_i = (int)L.size();
        // invneighboridx: atom -> slot (last image wins), slot 0 = central atom
        std::vector<int> inv(N, -1), nidx(nn_i + 1);
        inv[i1] = 0;
        nidx[0] = i1;
        for (int q = 0; q < nn_i; ++q) {
            inv[L[q].j] = q + 1;
            nidx[q + 1] = L[q].j;
        }
        std::vector<double> G(nsf, 0.0), dG((size_t)nsf * (nn_i + 1) * 3, 0.0);
        auto D = [&](int s, int slot, int d) -> double & { return dG[((size_t)s * (nn_i + 1) + slot) * 3 + d]; };
        const double xi = xyz[3 * i1], yi = xyz[3 * i1 + 1], zi = xyz[3 * i1 + 2];
        for (int s = 0; s < nsf; ++s) {
            const int k = e * nn->maxsf + s;
            const double rc = nn->rc[k];
            if (nn->sftype[k] == 2) {
                const double eta = nn->eta[k], rs = nn->rshift[k];
                for (int q = 0; q < nn_i; ++q) {
                    if (nn->e1[k] != L[q].elem) continue;
                    const double rij = L[q].r;
                    if (!(rij <= rc)) continue;
                    const double dx = -1.0 * (xi - L[q].x), dy = -1.0 * (yi - L[q].y), dz = -1.0 * (zi - L[q].z);
                    const double drx = -dx / rij, dry = -dy / rij, drz = -dz / rij;
                    double fc, t1;
                    getcutoff(nn->cutoff_type, nn->cutoff_alpha, rc, rij, fc, t1);
                    const double dfx = t1 * drx, dfy = t1 * dry, dfz = t1 * drz;
                    const double ex = std::exp(-1.0 * eta * (rij - rs) * (rij - rs));
                    G[s] += ex * fc;
                    const double tt1 = -2.0 * eta * (rij - rs) * ex * fc, tt2 = ex;
                    const int si = inv[i1], sj = inv[L[q].j];
                    D(s, si, 0) += drx * tt1 + tt2 * dfx;
                    D(s, sj, 0) += -drx * tt1 + tt2 * (-dfx);
                    D(s, si, 1) += dry * tt1 + tt2 * dfy;
                    D(s, sj, 1) += -dry * tt1 + tt2 * (-dfy);
                    D(s, si, 2) += drz * tt1 + tt2 * dfz;
                    D(s, sj, 2) += -drz * tt1 + tt2 * (-dfz);
                }
            } else if (nn->sftype[k] == 3) {
                const double eta = nn->eta[k], lam = nn->lambda[k], zeta = nn->zeta[k];
                const double rc2 = rc * rc;
                const double pnorm = std::pow(2.0, 1.0 - zeta), pzl = zeta * lam;
                const int a1 = nn->e1[k], a2 = nn->e2[k];
                double sum = 0.0;
                for (int q3 = 0; q3 < nn_i - 1; ++q3) {
                    const double rij = L[q3].r;
                    if (!(rij <= rc && (a1 == L[q3].elem || a2 == L[q3].elem))) continue;
                    const double r2ij = rij * rij;
                    double pfcij, pdfcij;
                    getcutoff(nn->cutoff_type, nn->cutoff_alpha, rc, rij, pfcij, pdfcij);
                    for (int q4 = q3 + 1; q4 < nn_i; ++q4) {
                        if (!((a1 == L[q3].elem && a2 == L[q4].elem) || (a2 == L[q3].elem && a1 == L[q4].elem)))
                            continue;
                        const double rik = L[q4].r;
                        if (!(rik <= rc)) continue;
                        double dxjk = L[q3].x - L[q4].x, dyjk = L[q3].y - L[q4].y, dzjk = L[q3].z - L[q4].z;
                        double rjk = dxjk * dxjk + dyjk * dyjk + dzjk * dzjk;
                        if (!(rjk <= rc2)) continue;
                        rjk = std::sqrt(rjk);
                        double rinv = 1.0 / rij / rik;
                        const double r2ik = rik * rik;
                        double dxij = xi - L[q3].x, dyij = yi - L[q3].y, dzij = zi - L[q3].z;
                        double dxik = xi - L[q4].x, dyik = yi - L[q4].y, dzik = zi - L[q4].z;
                        double pfcik, pdfcik, pfcjk, pdfcjk;
                        getcutoff(nn->cutoff_type, nn->cutoff_alpha, rc, rik, pfcik, pdfcik);
                        getcutoff(nn->cutoff_type, nn->cutoff_alpha, rc, rjk, pfcjk, pdfcjk);
                        double cost = (dxij * dxik + dyij * dyik + dzij * dzik) * rinv;
                        const double pfc = pfcij * pfcik * pfcjk;
                        const double pexp = std::exp(-eta * (r2ij + r2ik + rjk * rjk));
                        const double plam = 1.0 + lam * cost;
                        double fg = (plam <= 0.0) ? 0.0 : std::pow(plam, zeta - 1.0) * pexp;
                        sum += fg * plam * pfc;
                        fg = fg * pnorm;
                        rinv = rinv * pzl;
                        cost = cost * pzl;
                        const double p2el = 2.0 * eta * plam;
                        double p1 = pfc * (rinv - cost / r2ij - p2el) + pfcik * pfcjk * pdfcij * plam / rij;
                        double p2 = pfc * (rinv - cost / r2ik - p2el) + pfcij * pfcjk * pdfcik * plam / rik;
                        double p3 = pfc * (rinv + p2el) - pfcij * pfcik * pdfcjk * plam / rjk;
                        p1 *= fg; p2 *= fg; p3 *= fg;
                        dxij *= p1; dyij *= p1; dzij *= p1;
                        dxik *= p2; dyik *= p2; dzik *= p2;
                        dxjk *= p3; dyjk *= p3; dzjk *= p3;
                        const int si = inv[i1], sn = inv[L[q3].j], sm = inv[L[q4].j];
                        D(s, si, 0) += dxij + dxik; D(s, si, 1) += dyij + dyik; D(s, si, 2) += dzij + dzik;
                        D(s, sn, 0) += -dxij - dxjk; D(s, sn, 1) += -dyij - dyjk; D(s, sn, 2) += -dzij - dzjk;
                        D(s, sm, 0) += -dxik + dxjk; D(s, sm, 1) += -dyik + dyjk; D(s, sm, 2) += -dzik + dzjk;
                    }
                }
                G[s] = sum * pnorm;
            } else {
                return -5;  // symmetry-function type outside the G2/G3 subset
            }
        }
        // scaling, getshortatomic.f90:174-236
        for (int s = 0; s < nsf; ++s) {
            const int k = e * nn->maxsf + s;
            const double w = nn->smax[k] - nn->smin[k];
            if (nn->scalesym) {
                for (int q = 0; q <= nn_i; ++q)
                    for (int d = 0; d < 3; ++d) D(s, q, d) = D(s, q, d) / w * (nn->scmax - nn->scmin);
            }
            if (nn->centersym && !nn->scalesym) G[s] = G[s] - nn->savg[k];
            else if (nn->scalesym && !nn->centersym)
                G[s] = (G[s] - nn->smin[k]) / w * (nn->scmax - nn->scmin) + nn->scmin;
            else if (nn->scalesym && nn->centersym) G[s] = (G[s] - nn->savg[k]) / w;
            if (G_out) G_out[(size_t)i1 * nn->maxsf + s] = G[s];
        }
        // calconenn.f90:83-153
        const int nl = nn->nlayers, mx = nn->maxnodes;
        const int *nodes = nn->nodes + e * (nl + 1);
        const char *act = nn->act + (size_t)e * nl * mx;
        const double *w = nn->weights + (size_t)e * nn->maxweights;
        std::vector<double> val((nl + 1) * mx, 0.0), sumv((nl + 1) * mx, 0.0), dn((nl + 1) * mx, 0.0);
        int ic = 0;
        std::vector<int> woff(nl + 1, 0);  // offset of layer l weights
        for (int l = 1; l <= nl; ++l) {
            woff[l] = ic;
            for (int i3 = 0; i3 < nodes[l - 1]; ++i3)
                for (int i2 = 0; i2 < nodes[l]; ++i2) {
                    const double in = (l == 1) ? G[i3] : val[(l - 1) * mx + i3];
                    val[l * mx + i2] += w[ic++] * in;
                }
            for (int i2 = 0; i2 < nodes[l]; ++i2) {
                val[l * mx + i2] += w[ic++];
                if (nn->normnodes) val[l * mx + i2] /= (double)nodes[l - 1];
                sumv[l * mx + i2] = val[l * mx + i2];
                val[l * mx + i2] = act_f(act[(l - 1) * mx + i2], val[l * mx + i2]);
            }
        }
        const double eatom = val[nl * mx + 0];
        etot += eatom;
        if (eatom_out) eatom_out[i1] = eatom * kHa2eV;
        // getdnodes_values.f90:65-114
        for (int l = 1; l <= nl; ++l) {
            const double norm = nn->normnodes ? 1.0 / (double)nodes[l - 1] : 1.0;
            for (int i3 = 0; i3 < nodes[l]; ++i3)
                dn[l * mx + i3] = norm * act_d(act[(l - 1) * mx + i3], sumv[l * mx + i3], val[l * mx + i3]);
        }
        // forward-mode dE/dG, getshortatomic.f90:263-291
        std::vector<double> dEdG(nsf, 0.0);
        for (int s = 0; s < nsf; ++s) {
            std::vector<double> tprev(mx, 0.0), tcur(mx, 0.0);
            for (int i4 = 0; i4 < nodes[1]; ++i4) tprev[i4] = dn[1 * mx + i4] * w[s * nodes[1] + i4];
            for (int l = 2; l <= nl; ++l) {
                std::fill(tcur.begin(), tcur.end(), 0.0);
                for (int i3 = 0; i3 < nodes[l]; ++i3)
                    for (int i4 = 0; i4 < nodes[l - 1]; ++i4)
                        tcur[i3] += dn[l * mx + i3] * w[woff[l] + i4 * nodes[l] + i3] * tprev[i4];
                tprev = tcur;
            }
            dEdG[s] = tprev[0];
        }
        // force scatter, getshortatomic.f90:296-322
        for (int s = 0; s < nsf; ++s)
            for (int q = 0; q <= nn_i; ++q)
                for (int d = 0; d < 3; ++d) F[3 * nidx[q] + d] -= dEdG[s] * D(s, q, d);
    }
    if (nn->remove_atom_energies)
        for (int a = 0; a < N; ++a) etot += nn->atom_energy[elem[a]];
    *energy_ev = etot * kHa2eV;
    const double habohr2evang = kHa2eV * kAng2Bohr;
    for (int k = 0; k < 3 * N; ++k) forces[k] = F[k] * habohr2evang;
    return 0;
}

}  // extern "C"
