// gw_setup.cpp -- host-side set-up of a context: the reference's material
// model folded into small coefficient tables, the advection index lists and
// the ROCK2 stage rule.  Compiled with -ffp-contract=off so every comparison
// that classifies a cell rounds exactly as the reference's scalar code.
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "gw_internal.h"
#include "rock2_table.h"

namespace {

// src/physics.jl:102-125 (homogeneous == one layer)
int layer_of(const gw_ctx *c, double z) {
    int n = (int)c->depths.size();
    for (int i = 0; i < n; ++i)
        if (z <= c->depths[i]) return i;
    return n - 1;
}

// src/physics.jl:199-233 get_thermal_conductivity
double mat_k(const gw_ctx *c, double x, double y, double z) {
    double k = c->k_layers[layer_of(c, z)];
    for (const GwBorehole &b : c->bh) {
        double dx = x - b.xc, dy = y - b.yc;
        double r_sq = dx * dx + dy * dy;
        if (r_sq > b.r_backfill_sq) continue;
        if (z <= b.h) {
            if (r_sq < b.r_inner * b.r_inner) k = c->k_water;
            else if (r_sq < b.r_and_t_inner_sq) k = c->k_insulating;
            else if (r_sq < b.r_outer_sq) k = c->k_water;
            else if (r_sq < b.r_and_t_outer_sq) k = (z <= b.insulation_depth) ? c->k_insulating : c->k_steel;
            else k = c->k_backfill;
        } else if (z <= b.h + 3) {
            k = c->k_steel;
        }
    }
    return k;
}

// src/physics.jl:243-274 get_volumetric_heat_capacity
double mat_rhoc(const gw_ctx *c, double x, double y, double z) {
    double rc = c->rhoc_layers[layer_of(c, z)];
    for (const GwBorehole &b : c->bh) {
        double dx = x - b.xc, dy = y - b.yc;
        double r_sq = dx * dx + dy * dy;
        if (r_sq > b.r_and_t_outer_sq) continue;
        if (z <= b.h) {
            if (r_sq < b.r_inner * b.r_inner) rc = c->rho_c_water;
            else if (r_sq < b.r_and_t_inner_sq) rc = c->rho_c_insulating;
            else if (r_sq < b.r_outer_sq) rc = c->rho_c_water;
            else rc = (z <= b.insulation_depth) ? c->rho_c_insulating : c->rho_c_steel;
        } else if (z <= b.h + 3) {
            rc = c->rho_c_steel;
        }
    }
    return rc;
}

bool strictly_increasing(const double *g, int n) {
    for (int i = 0; i + 1 < n; ++i)
        if (!(g[i + 1] > g[i])) return false;
    return true;
}

}  // namespace

// Column profiles: columns whose (k, rho_c) sequences over the z-classes
// agree share their z coefficients; ids in order of first appearance
// (i, then j).
void gw_build_profiles(gw_ctx *c) {
    std::vector<int> rep(c->n_zclass, -1);
    for (int k = 0; k < c->nz; ++k)
        if (rep[c->zclass[k]] < 0) rep[c->zclass[k]] = k;
    // column profiles: columns whose (k, rho_c) sequences over z-classes agree
    c->colprof.assign((size_t)c->nx * c->ny, 0);
    std::map<std::vector<double>, int> prof;
    for (int i = 0; i < c->nx; ++i)
        for (int j = 0; j < c->ny; ++j) {
            std::vector<double> key;
            key.reserve(2 * c->n_zclass);
            for (int zc = 0; zc < c->n_zclass; ++zc) {
                double z = c->gz[rep[zc]];
                key.push_back(mat_k(c, c->gx[i], c->gy[j], z));
                key.push_back(mat_rhoc(c, c->gx[i], c->gy[j], z));
            }
            auto it = prof.find(key);
            int id;
            if (it == prof.end()) {
                id = (int)prof.size();
                prof.emplace(std::move(key), id);
            } else {
                id = it->second;
            }
            c->colprof[(size_t)i * c->ny + j] = id;
        }
    c->n_profiles = (int)prof.size();
}

// Builds everything create_cache does on the host (src/cache.jl:9-44,55-65)
// plus the z-classes: maximal sets of levels on which every depth comparison
// of the material model (layers, z <= h, z <= h + 3, z <= insulation_depth)
// has the same outcome, so materials are exact per (z-class, i, j).
int gw_setup_host(gw_ctx *c, const gw_desc *d) {
    if (!d) return gw_fail(GW_ERR_ARG, "desc is NULL");
    if (d->nx < 2 || d->ny < 2 || d->nz < 2)
        return gw_fail(GW_ERR_ARG, "grids need at least 2 points in each direction");
    if (d->nx > 65536 || d->ny > 65536 || d->nz > (1 << 24))
        return gw_fail(GW_ERR_ARG, "grid too large");
    if (!d->gridx || !d->gridy || !d->gridz) return gw_fail(GW_ERR_ARG, "grid pointer is NULL");
    if (!strictly_increasing(d->gridx, d->nx) || !strictly_increasing(d->gridy, d->ny) ||
        !strictly_increasing(d->gridz, d->nz))
        return gw_fail(GW_ERR_ARG, "grids must be strictly increasing");
    if (d->n_boreholes < 1 || !d->boreholes) return gw_fail(GW_ERR_ARG, "need at least one borehole");
    if (d->materials.n_layers < 1 || !d->materials.k_rock_layers || !d->materials.rho_c_rock_layers ||
        !d->materials.layer_depths)
        return gw_fail(GW_ERR_ARG, "materials need at least one rock layer");
    if (d->inlet_kind != GW_INLET_CONSTANT && d->inlet_kind != GW_INLET_HEAT_EXCHANGER &&
        d->inlet_kind != GW_INLET_SCHEDULE && d->inlet_kind != GW_INLET_EXPRESSION)
        return gw_fail(GW_ERR_UNSUPPORTED, "inlet kind must be GW_INLET_CONSTANT, GW_INLET_HEAT_EXCHANGER, "
                                           "GW_INLET_SCHEDULE or GW_INLET_EXPRESSION (CustomInlet closures "
                                           "cannot cross the C ABI)");
    if (d->precision != GW_PREC_FP64 && d->precision != GW_PREC_MIXED)
        return gw_fail(GW_ERR_ARG, "precision must be GW_PREC_FP64 or GW_PREC_MIXED");

    c->nx = d->nx; c->ny = d->ny; c->nz = d->nz;
    c->gx.assign(d->gridx, d->gridx + d->nx);
    c->gy.assign(d->gridy, d->gridy + d->ny);
    c->gz.assign(d->gridz, d->gridz + d->nz);
    c->precision = d->precision;
    c->inlet_kind = d->inlet_kind;
    c->inlet_param = d->inlet_param;
    const gw_material_desc &m = d->materials;
    c->k_layers.assign(m.k_rock_layers, m.k_rock_layers + m.n_layers);
    c->rhoc_layers.assign(m.rho_c_rock_layers, m.rho_c_rock_layers + m.n_layers);
    c->depths.assign(m.layer_depths, m.layer_depths + m.n_layers);
    c->k_water = m.k_water; c->rho_c_water = m.rho_c_water;
    c->k_steel = m.k_steel; c->rho_c_steel = m.rho_c_steel;
    c->k_insulating = m.k_insulating; c->rho_c_insulating = m.rho_c_insulating;
    c->k_backfill = m.k_backfill; c->rho_c_backfill = m.rho_c_backfill;

    // src/physics.jl:48-59
    const double pi = 3.141592653589793;
    c->nbh = d->n_boreholes;
    c->bh.resize(c->nbh);
    for (int b = 0; b < c->nbh; ++b) {
        const gw_borehole_desc &p = d->boreholes[b];
        GwBorehole &o = c->bh[b];
        o.xc = p.xc; o.yc = p.yc; o.h = p.h; o.r_inner = p.r_inner; o.t_inner = p.t_inner;
        o.r_outer = p.r_outer; o.t_outer = p.t_outer; o.r_backfill = p.r_backfill;
        o.mdot = p.mdot; o.insulation_depth = p.insulation_depth;
        double rti = o.r_inner + o.t_inner;
        o.r_and_t_inner_sq = rti * rti;
        o.r_outer_sq = o.r_outer * o.r_outer;
        double rto = o.r_outer + o.t_outer;
        o.r_and_t_outer_sq = rto * rto;
        o.r_backfill_sq = o.r_backfill * o.r_backfill;
        double A_inner = pi * (o.r_inner * o.r_inner);
        double A_outer = pi * o.r_outer_sq - pi * o.r_and_t_inner_sq;
        const double rho_water = 998.2;
        o.v_inner = o.mdot / (A_inner * rho_water);
        o.v_outer = o.mdot / (A_outer * rho_water);
    }

    // src/solver.jl:474-488 with src/physics.jl:134-149
    double dzmin = INFINITY;
    for (int k = 0; k + 1 < c->nz; ++k) dzmin = std::fmin(dzmin, c->gz[k + 1] - c->gz[k]);
    double dmax = 0.0;
    for (int i = 0; i < m.n_layers; ++i) dmax = std::fmax(dmax, c->k_layers[i] / c->rhoc_layers[i]);
    dmax = std::fmax(dmax, c->k_water / c->rho_c_water);
    dmax = std::fmax(dmax, c->k_steel / c->rho_c_steel);
    dmax = std::fmax(dmax, c->k_insulating / c->rho_c_insulating);
    dmax = std::fmax(dmax, c->k_backfill / c->rho_c_backfill);
    c->eigen_estimate = 8 * dmax / (dzmin * dzmin);

    // z-classes
    c->zclass.assign(c->nz, 0);
    std::map<std::vector<int>, int> sig;
    std::vector<int> rep;   // representative level per class
    for (int k = 0; k < c->nz; ++k) {
        double z = c->gz[k];
        std::vector<int> s;
        s.push_back(layer_of(c, z));
        for (const GwBorehole &b : c->bh) {
            s.push_back(z <= b.h);
            s.push_back(z <= b.h + 3);
            s.push_back(z <= b.insulation_depth);
        }
        auto it = sig.find(s);
        if (it == sig.end()) {
            int id = (int)rep.size();
            sig.emplace(s, id);
            rep.push_back(k);
            c->zclass[k] = id;
        } else {
            c->zclass[k] = it->second;
        }
    }
    c->n_zclass = (int)rep.size();

    // column profiles: on the host path here, else grouped on the GPU
    // (gw_setup_dev.cu)
    if (c->host_setup) gw_build_profiles(c);

    // src/cache.jl:9-44 create_advection_index_lists
    std::vector<int> ii, ij, ib, oi, oj, ob;
    for (int b = 0; b < c->nbh; ++b) {
        const GwBorehole &bh = c->bh[b];
        for (int i = 0; i < c->nx; ++i)
            for (int j = 0; j < c->ny; ++j) {
                double dx = c->gx[i] - bh.xc, dy = c->gy[j] - bh.yc;
                double r_sq = dx * dx + dy * dy;
                double rti = bh.r_inner + bh.t_inner;
                if (r_sq < bh.r_inner * bh.r_inner) {
                    ii.push_back(i); ij.push_back(j); ib.push_back(b);
                } else if (rti * rti <= r_sq && r_sq < bh.r_outer * bh.r_outer) {
                    oi.push_back(i); oj.push_back(j); ob.push_back(b);
                }
            }
    }
    c->n_inner = (int)ii.size();
    c->n_outer = (int)oi.size();
    c->pipe_i = ii; c->pipe_i.insert(c->pipe_i.end(), oi.begin(), oi.end());
    c->pipe_j = ij; c->pipe_j.insert(c->pipe_j.end(), oj.begin(), oj.end());
    c->pipe_b = ib; c->pipe_b.insert(c->pipe_b.end(), ob.begin(), ob.end());
    double max_h = -INFINITY;
    for (const GwBorehole &b : c->bh) max_h = std::fmax(max_h, b.h);
    int cz = 0;
    for (int k = 0; k < c->nz; ++k)
        if (c->gz[k] <= max_h) ++cz;
    c->countz = cz;
    return GW_OK;
}

// Coefficients of the 3-point operators A_x, A_y, A_z in the form
//   (A phi)_l = cp_l (phi_{l+1} - phi_l) - cm_l (phi_l - phi_{l-1})
// with the reference's face conductivity (k_l + k_{l+-1})/2, its spacings and
// its Neumann ends (src/solver.jl:34-109): cm = 0 at the first point, cp = 0
// at the last, and the end spacing mirrored.
void gw_build_coefs(const gw_ctx *c, std::vector<double> &cxm, std::vector<double> &cxp,
                    std::vector<double> &cym, std::vector<double> &cyp,
                    std::vector<double> &czm, std::vector<double> &czp) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, nzc = c->n_zclass;
    std::vector<int> rep(nzc, -1);
    for (int k = 0; k < nz; ++k)
        if (rep[c->zclass[k]] < 0) rep[c->zclass[k]] = k;
    // material values per (zc, i, j)
    std::vector<double> K((size_t)nzc * nx * ny), R((size_t)nzc * nx * ny);
    for (int zc = 0; zc < nzc; ++zc)
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                double z = c->gz[rep[zc]];
                size_t q = ((size_t)zc * nx + i) * ny + j;
                K[q] = mat_k(c, c->gx[i], c->gy[j], z);
                R[q] = mat_rhoc(c, c->gx[i], c->gy[j], z);
            }
    auto KI = [&](int zc, int i, int j) { return K[((size_t)zc * nx + i) * ny + j]; };
    auto RI = [&](int zc, int i, int j) { return R[((size_t)zc * nx + i) * ny + j]; };
    auto coef = [](const double *g, int n, int l, double kc, double km, double kp, double rc,
                   double *cm, double *cp) {
        double dp = (l == n - 1) ? (g[l] - g[l - 1]) : (g[l + 1] - g[l]);
        double dm = (l == 0) ? dp : (g[l] - g[l - 1]);
        double mid = (dp + dm) * 0.5;
        *cp = (l == n - 1) ? 0.0 : (kp + kc) * 0.5 / dp / mid / rc;
        *cm = (l == 0) ? 0.0 : (kc + km) * 0.5 / dm / mid / rc;
    };
    cxm.assign((size_t)nzc * ny * nx, 0); cxp.assign((size_t)nzc * ny * nx, 0);
    cym.assign((size_t)nzc * nx * ny, 0); cyp.assign((size_t)nzc * nx * ny, 0);
    for (int zc = 0; zc < nzc; ++zc)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int ipl = i == nx - 1 ? i : i + 1, imi = i == 0 ? i : i - 1;
                size_t q = ((size_t)zc * ny + j) * nx + i;
                coef(c->gx.data(), nx, i, KI(zc, i, j), KI(zc, imi, j), KI(zc, ipl, j), RI(zc, i, j),
                     &cxm[q], &cxp[q]);
            }
    for (int zc = 0; zc < nzc; ++zc)
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                int jpl = j == ny - 1 ? j : j + 1, jmi = j == 0 ? j : j - 1;
                size_t q = ((size_t)zc * nx + i) * ny + j;
                coef(c->gy.data(), ny, j, KI(zc, i, j), KI(zc, i, jmi), KI(zc, i, jpl), RI(zc, i, j),
                     &cym[q], &cyp[q]);
            }
    // z: one representative column per profile
    std::vector<int> prof_i(c->n_profiles, -1), prof_j(c->n_profiles, -1);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            int p = c->colprof[(size_t)i * ny + j];
            if (prof_i[p] < 0) { prof_i[p] = i; prof_j[p] = j; }
        }
    czm.assign((size_t)c->n_profiles * nz, 0); czp.assign((size_t)c->n_profiles * nz, 0);
    for (int p = 0; p < c->n_profiles; ++p) {
        int i = prof_i[p], j = prof_j[p];
        for (int k = 0; k < nz; ++k) {
            int kpl = k == nz - 1 ? k : k + 1, kmi = k == 0 ? k : k - 1;
            coef(c->gz.data(), nz, k, KI(c->zclass[k], i, j), KI(c->zclass[kmi], i, j),
                 KI(c->zclass[kpl], i, j), RI(c->zclass[k], i, j), &czm[(size_t)p * nz + k],
                 &czp[(size_t)p * nz + k]);
        }
    }
}

// Tables of the adjoint.  The coefficients above are cp_l = (k_l + k_{l+1}) wp_l
// and cm_l = (k_l + k_{l-1}) wm_l with wp_l = 0.5 / dp / mid / rho_c_l and
// wm_l = 0.5 / dm / mid / rho_c_l (0 at the Neumann ends), so the derivative of
// lambda^T A phi with respect to the conductivity of one cell is a sum of face
// terms D = (phi_{l+1} - phi_l) (lambda_l wp_l - lambda_{l+1} wm_{l+1}) over
// the cell's two faces.  rock[(zc * nx + i) * ny + j] = 1 where the cell's
// conductivity is its rock layer's (src/physics.jl:199-233: no borehole
// within r_backfill overrides it at that depth), i.e. where it depends on
// the layer conductivity; layer[k] = the rock layer of level k.
void gw_build_adjoint_tables(const gw_ctx *c, std::vector<double> &wxm, std::vector<double> &wxp,
                             std::vector<double> &wym, std::vector<double> &wyp,
                             std::vector<double> &wzm, std::vector<double> &wzp,
                             std::vector<unsigned char> &rock, std::vector<int> &layer) {
    const int nx = c->nx, ny = c->ny, nz = c->nz, nzc = c->n_zclass;
    std::vector<int> rep(nzc, -1);
    for (int k = 0; k < nz; ++k)
        if (rep[c->zclass[k]] < 0) rep[c->zclass[k]] = k;
    std::vector<double> R((size_t)nzc * nx * ny);
    rock.assign((size_t)nzc * nx * ny, 0);
    for (int zc = 0; zc < nzc; ++zc)
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                double z = c->gz[rep[zc]];
                size_t q = ((size_t)zc * nx + i) * ny + j;
                R[q] = mat_rhoc(c, c->gx[i], c->gy[j], z);
                bool r = true;
                for (const GwBorehole &b : c->bh) {
                    double dx = c->gx[i] - b.xc, dy = c->gy[j] - b.yc;
                    double r_sq = dx * dx + dy * dy;
                    if (r_sq > b.r_backfill_sq) continue;
                    if (z <= b.h || z <= b.h + 3) r = false;
                }
                rock[q] = r ? 1 : 0;
            }
    auto RI = [&](int zc, int i, int j) { return R[((size_t)zc * nx + i) * ny + j]; };
    auto unit = [](const double *g, int n, int l, double rc, double *wm, double *wp) {
        double dp = (l == n - 1) ? (g[l] - g[l - 1]) : (g[l + 1] - g[l]);
        double dm = (l == 0) ? dp : (g[l] - g[l - 1]);
        double mid = (dp + dm) * 0.5;
        *wp = (l == n - 1) ? 0.0 : 0.5 / dp / mid / rc;
        *wm = (l == 0) ? 0.0 : 0.5 / dm / mid / rc;
    };
    wxm.assign((size_t)nzc * ny * nx, 0); wxp.assign((size_t)nzc * ny * nx, 0);
    wym.assign((size_t)nzc * nx * ny, 0); wyp.assign((size_t)nzc * nx * ny, 0);
    for (int zc = 0; zc < nzc; ++zc)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t q = ((size_t)zc * ny + j) * nx + i;
                unit(c->gx.data(), nx, i, RI(zc, i, j), &wxm[q], &wxp[q]);
            }
    for (int zc = 0; zc < nzc; ++zc)
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                size_t q = ((size_t)zc * nx + i) * ny + j;
                unit(c->gy.data(), ny, j, RI(zc, i, j), &wym[q], &wyp[q]);
            }
    std::vector<int> prof_i(c->n_profiles, -1), prof_j(c->n_profiles, -1);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            int p = c->colprof[(size_t)i * ny + j];
            if (prof_i[p] < 0) { prof_i[p] = i; prof_j[p] = j; }
        }
    wzm.assign((size_t)c->n_profiles * nz, 0); wzp.assign((size_t)c->n_profiles * nz, 0);
    for (int p = 0; p < c->n_profiles; ++p)
        for (int k = 0; k < nz; ++k)
            unit(c->gz.data(), nz, k, RI(c->zclass[k], prof_i[p], prof_j[p]), &wzm[(size_t)p * nz + k],
                 &wzp[(size_t)p * nz + k]);
    layer.assign(nz, 0);
    for (int k = 0; k < nz; ++k) layer[k] = layer_of(c, c->gz[k]);
}

// LU factors of (I - h A) for every (z-class, line) of one direction, in the
// scaled form used by the line kernels (src/solver.jl:208-218 elimination).
void gw_build_factors(const gw_ctx *c, double h, int dir, const std::vector<double> &cm,
                      const std::vector<double> &cp, std::vector<double> &a,
                      std::vector<double> &ib, std::vector<double> &cu) {
    const int N = dir == GW_DIR_X ? c->nx : c->ny;
    const int nl = dir == GW_DIR_X ? c->ny : c->nx;
    const size_t tot = (size_t)c->n_zclass * nl * N;
    a.assign(tot, 0); ib.assign(tot, 0); cu.assign(tot, 0);
    for (size_t line = 0; line < (size_t)c->n_zclass * nl; ++line) {
        const double *m_ = &cm[line * N];
        const double *p_ = &cp[line * N];
        double dprev = 0.0, uprev = 0.0;
        for (int l = 0; l < N; ++l) {
            double lower = -h * m_[l];
            double diag = 1.0 + h * (m_[l] + p_[l]);
            double upper = -h * p_[l];
            if (l > 0) diag -= (lower / dprev) * uprev;
            a[line * N + l] = (l > 0) ? lower : 0.0;
            ib[line * N + l] = 1.0 / diag;
            cu[line * N + l] = upper / diag;
            dprev = diag;
            uprev = upper;
        }
    }
}

// Per (z-class, line, row) of one line direction: the explicit sweep of the
// other direction, (I + h A_e), folded with the forward elimination of
// (I - h A_line):  y_l = e0 x_c + ep x_+ + em x_- - a y_{l-1}  with
// e0 = (1 - h (cp + cm)) ib, ep = h cp ib, em = h cm ib, a = lower ib.
// dir X: x-lines (zc, j, i), explicit y coefficients [zc][i][j];
// dir Y: y-lines (zc, i, j), explicit x coefficients [zc][j][i].
void gw_build_half_table(const gw_ctx *c, double h, int dir, const std::vector<double> &ecm,
                         const std::vector<double> &ecp, const std::vector<double> &a,
                         const std::vector<double> &ib, std::vector<double> &out4) {
    const int nl = dir == GW_DIR_X ? c->ny : c->nx;
    const int N = dir == GW_DIR_X ? c->nx : c->ny;
    out4.assign((size_t)c->n_zclass * nl * N * 4, 0.0);
    for (int zc = 0; zc < c->n_zclass; ++zc)
        for (int m = 0; m < nl; ++m)
            for (int l = 0; l < N; ++l) {
                const size_t q = ((size_t)zc * nl + m) * N + l;
                // explicit coefficient table index of the same cell
                const size_t e = ((size_t)zc * N + l) * nl + m;
                const double cm = ecm[e], cp = ecp[e], g = ib[q];
                out4[4 * q + 0] = (1.0 - h * (cp + cm)) * g;
                out4[4 * q + 1] = h * cp * g;
                out4[4 * q + 2] = h * cm * g;
                out4[4 * q + 3] = a[q] * g;
            }
}

// Stage count: the smallest s >= 3 (at least one recurrence stage) whose
// stability interval l_s covers |dt| * eigen_est, capped at max_stages.
int gw_rock2_choose(double dt, double eigen_est, int max_stages, int *s, int *covered) {
    if (max_stages < 3) return gw_fail(GW_ERR_ARG, "max_stages must be >= 3");
    int cap = max_stages < GW_ROCK2_S_MAX ? max_stages : GW_ROCK2_S_MAX;
    double x = std::fabs(dt) * eigen_est;
    for (int k = 3; k <= cap; ++k)
        if (gw_rock2_l[k - 2] >= x) {
            *s = k;
            *covered = 1;
            return GW_OK;
        }
    *s = cap;
    *covered = 0;
    return GW_OK;
}

void gw_rock2_coefs(int s, const double **mu, const double **nu, const double **kappa,
                    double *sigma, double *tau) {
    int o = gw_rock2_off[s - 2];
    *mu = gw_rock2_mu + o;
    *nu = gw_rock2_nu + o;
    *kappa = gw_rock2_kappa + o;
    *sigma = gw_rock2_sigma[s - 2];
    *tau = gw_rock2_tau[s - 2];
}
