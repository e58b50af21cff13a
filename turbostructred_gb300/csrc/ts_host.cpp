// Host-side set-up of the GB300-native explicit FVM step: grid geometry,
// configuration checks, error reporting and the synthetic benchmark
// scenarios.  Pure C++ (no CUDA), compiled into the same shared library.
#include <cmath>
#include <cstring>
#include <string>

#include "ts_internal.h"

namespace ts {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

ts_status fail(ts_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

// One axis of Grid::InitLocal (grid.h:164-218): cell centres are accumulated
// cell by cell, xc += 0.5*h*(1+q), starting half a step inside the first
// ghost layer, so the device sees exactly the reference's coordinates.
static void axis_grid(const ts_config& c, int a, int n, double L, std::vector<double>& X,
                      std::vector<double>& H) {
    const int g = 1;
    X.assign(n + 2 * g, 0.0);
    H.assign(n + 2 * g, 0.0);
    std::vector<double> pos, q;
    std::vector<int> nc;
    if (c.n_blocks[a] <= 0 || c.blocks[a] == nullptr) {
        pos.push_back(0.0); q.push_back(1.0); nc.push_back(-1);
    } else {
        for (int b = 0; b < c.n_blocks[a]; ++b) {
            pos.push_back(c.blocks[a][b].pos);
            q.push_back(c.blocks[a][b].q_com);
            nc.push_back(c.blocks[a][b].n_cells);
        }
    }
    pos.push_back(L); q.push_back(1.0); nc.push_back(-1);  // closing node (grid.h:165)

    double stp = 1.0;
    if (nc[0] < 1) {
        stp = L / n;
        nc[0] = n;
    } else {
        double len = pos[1] - pos[0];
        if (q[0] == 1.0) stp = len / nc[0];
        else stp = len * (1.0 - q[0]) / (1.0 - std::pow(q[0], nc[0]));
    }
    double xc = -(g * stp) + 0.5 * stp;
    int ci = 0;
    for (; ci < g; ++ci) { X[ci] = xc; H[ci] = stp; xc += stp; }
    for (size_t b = 1; b < pos.size(); ++b) {
        const double qb = q[b - 1];
        for (int i = 0; i < nc[b - 1]; ++i) {
            X[ci + i] = xc;
            H[ci + i] = stp;
            xc += 0.5 * stp * (1.0 + qb);
            stp *= qb;
        }
        ci += nc[b - 1];
        if (nc[b] > 0) {
            double len = pos[b + 1] - pos[b];
            if (q[b] == 1.0) stp = len / nc[b];
            else stp = len * (1.0 - q[b]) / (1.0 - std::pow(q[b], nc[b]));
            xc = pos[b] + 0.5 * stp;
        }
    }
    for (int i = 0; i < g; ++i) { X[ci + i] = xc; H[ci + i] = stp; xc += stp; }
}

ts_status validate_config(const ts_config& c, std::string& err) {
    if (c.abi_version != TS_FVM_ABI_VERSION) { err = "ts_config.abi_version mismatch"; return TS_ERR_INVALID; }
    if (c.n_dims < 1 || c.n_dims > 3) { err = "n_dims must be 1, 2 or 3"; return TS_ERR_INVALID; }
    const int n[3] = {c.nx, c.ny, c.nz};
    for (int a = 0; a < c.n_dims; ++a) {
        if (n[a] < 2) { err = "each active axis needs at least 2 cells"; return TS_ERR_INVALID; }
        if (c.n_blocks[a] < 0 || c.n_blocks[a] > 64) { err = "n_blocks out of range"; return TS_ERR_INVALID; }
        if (c.n_blocks[a] > 0) {
            if (!c.blocks[a]) { err = "blocks pointer is NULL"; return TS_ERR_INVALID; }
            long long tot = 0;
            for (int b = 0; b < c.n_blocks[a]; ++b) tot += c.blocks[a][b].n_cells;
            if (tot != n[a]) { err = "block cell counts do not sum to the axis size"; return TS_ERR_INVALID; }
        }
        if (!(c.length[a] > 0.0)) { err = "domain lengths must be positive"; return TS_ERR_INVALID; }
    }
    if ((long long)c.nx * (c.n_dims > 1 ? c.ny : 1) * (c.n_dims > 2 ? c.nz : 1) > (1LL << 31)) {
        err = "grid too large"; return TS_ERR_INVALID;
    }
    if (!(c.gamma > 1.0)) { err = "gamma must exceed 1"; return TS_ERR_INVALID; }
    if (c.eos != TS_EOS_IDEAL_GAS && c.eos != TS_EOS_STIFFENED_GAS) { err = "unknown eos"; return TS_ERR_INVALID; }
    if (c.eos == TS_EOS_STIFFENED_GAS && !(c.p_inf >= 0.0)) { err = "p_inf must be >= 0"; return TS_ERR_INVALID; }
    if (c.reconstruction < 0 || c.reconstruction > 3) { err = "unknown reconstruction"; return TS_ERR_INVALID; }
    if (c.limiter < 0 || c.limiter > 1) { err = "unknown limiter"; return TS_ERR_INVALID; }
    if (c.riemann_solver == TS_RS_GODUNOV) {
        if (c.precision != TS_PRECISION_FP64) {
            err = "the exact Godunov solver runs on the FP64 path"; return TS_ERR_UNSUPPORTED;
        }
        if (c.eos != TS_EOS_IDEAL_GAS) {
            err = "the exact Godunov solver is built for the ideal-gas EOS"; return TS_ERR_UNSUPPORTED;
        }
    }
    if (c.riemann_solver == TS_RS_NONE) {
        // InitializeMethod asserts a solver was chosen (ExplicitRungeKuttaFVM.h:43)
        err = "no Riemann solver chosen"; return TS_ERR_INVALID;
    }
    if (c.riemann_solver != TS_RS_ROE_PIKE && c.riemann_solver != TS_RS_HLLC && c.riemann_solver != TS_RS_GODUNOV) {
        err = "unknown riemann_solver"; return TS_ERR_INVALID;
    }
    if (!(c.cfl > 0.0)) { err = "cfl must be positive"; return TS_ERR_INVALID; }
    if (!(c.eps >= 0.0)) { err = "eps must be >= 0"; return TS_ERR_INVALID; }
    for (int s = 0; s < 2 * c.n_dims; ++s) {
        if (c.periodic[s / 2]) continue;
        if (c.bc[s].type < TS_BC_WALL || c.bc[s].type > TS_BC_NATURAL) { err = "unknown boundary condition"; return TS_ERR_INVALID; }
    }
    if (c.n_bc_kinds < 0 || c.n_bc_kinds > TS_MAX_BC_KINDS) { err = "n_bc_kinds out of range"; return TS_ERR_INVALID; }
    for (int k = 0; k < c.n_bc_kinds; ++k)
        if (c.bc_kinds[k].type < TS_BC_WALL || c.bc_kinds[k].type > TS_BC_NATURAL) {
            err = "unknown boundary condition in bc_kinds"; return TS_ERR_INVALID;
        }
    for (int s = 0; s < 6; ++s) {
        if (!c.bc_marker[s]) continue;
        if (s >= 2 * c.n_dims || c.periodic[s / 2]) {
            err = "bc_marker on a periodic or inactive side"; return TS_ERR_INVALID;
        }
        const long long nf = side_faces(c, s);
        for (long long f = 0; f < nf; ++f)
            if (c.bc_marker[s][f] >= c.n_bc_kinds) { err = "bc_marker entry beyond n_bc_kinds"; return TS_ERR_INVALID; }
    }
    if (c.precision != TS_PRECISION_FP64 && c.precision != TS_PRECISION_MIXED) { err = "unknown precision"; return TS_ERR_INVALID; }
    if (!(c.viscosity >= 0.0) || !std::isfinite(c.viscosity)) { err = "viscosity must be finite and >= 0"; return TS_ERR_INVALID; }
    if ((c.viscous || c.viscosity != 0.0) && c.precision != TS_PRECISION_FP64) {
        // the viscosity enters the spectral radius even without viscous fluxes
        err = "viscous flow (or a nonzero viscosity) runs on the FP64 path"; return TS_ERR_UNSUPPORTED;
    }
    return TS_OK;
}

ts_status build_grid(const ts_config& c, HostGrid& g, std::string& err) {
    ts_status s = validate_config(c, err);
    if (s != TS_OK) return s;
    axis_grid(c, 0, c.nx, c.length[0], g.x, g.hx);
    if (c.n_dims > 1) axis_grid(c, 1, c.ny, c.length[1], g.y, g.hy);
    else { g.y.assign(1, 0.0); g.hy.assign(1, 1.0); }   // grid.h:343
    if (c.n_dims > 2) axis_grid(c, 2, c.nz, c.length[2], g.z, g.hz);
    else { g.z.assign(1, 0.0); g.hz.assign(1, 1.0); }   // grid.h:344
    return TS_OK;
}

Layout make_layout(const ts_config& c) {
    Layout L;
    L.nd = c.n_dims;
    L.nx = c.nx;
    L.ny = c.n_dims > 1 ? c.ny : 1;
    L.nz = c.n_dims > 2 ? c.nz : 1;
    L.gx = GHOST;
    L.gy = c.n_dims > 1 ? GHOST : 0;
    L.gz = c.n_dims > 2 ? GHOST : 0;
    L.ex = L.nx + 2 * L.gx;
    L.ey = L.ny + 2 * L.gy;
    L.ez = L.nz + 2 * L.gz;
    L.px = (L.ex + 7) & ~7;
    long long p = (long long)L.px * L.ey * L.ez;
    L.plane = (p + 63) & ~63LL;
    return L;
}

Phys make_phys(const ts_config& c) {
    Phys p;
    std::memset(&p, 0, sizeof p);
    p.nd = c.n_dims;
    p.recon = c.reconstruction;
    p.limiter = c.limiter;
    p.solver = c.riemann_solver;
    p.eos = c.eos;
    for (int a = 0; a < 3; ++a) p.periodic[a] = (a < c.n_dims) ? (c.periodic[a] != 0) : 1;
    p.gamma = c.gamma;
    p.p_inf = c.eos == TS_EOS_STIFFENED_GAS ? c.p_inf : 0.0;
    p.eps = c.eps;
    p.cfl = c.cfl;
    for (int id = 0; id < kBcIds; ++id) {
        const bool side = id < 6;
        if (!side && id - 6 >= c.n_bc_kinds) continue;
        const ts_bc_config& b = side ? c.bc[id] : c.bc_kinds[id - 6];
        p.bc.type[id] = b.type;
        p.bc.density[id] = b.density;
        for (int a = 0; a < 3; ++a) p.bc.vel[id][a] = b.velocity[a];
        p.bc.pstatic[id] = b.pstatic;
    }
    // device marker arrays are set by their owner after the upload
    for (int s = 0; s < 6; ++s) p.bc.mark[s] = nullptr;
    p.viscous = c.viscous != 0;
    p.visc = c.viscosity;
    p.force = c.external_force != 0;
    p.accel = c.uniform_acceleration != 0;
    for (int a = 0; a < 3; ++a) {
        p.sigma[a] = p.force ? c.sigma[a] : 0.0;
        p.g[a] = p.accel ? c.acceleration[a] : 0.0;
    }
    return p;
}

}  // namespace ts

using namespace ts;

extern "C" {

const char* ts_last_error(void) { return g_last_error.c_str(); }

const char* ts_status_string(ts_status s) {
    switch (s) {
    case TS_OK: return "ok";
    case TS_ERR_INVALID: return "invalid argument";
    case TS_ERR_UNSUPPORTED: return "unsupported";
    case TS_ERR_CUDA: return "CUDA error";
    case TS_ERR_NO_MEMORY: return "out of memory";
    case TS_ERR_NUMERIC: return "numerical failure";
    case TS_ERR_TIMEOUT: return "timeout";
    case TS_ERR_BUSY: return "busy";
    case TS_ERR_NOT_FOUND: return "not found";
    }
    return "unknown status";
}

ts_status ts_grid_coordinates(const ts_config* cfg, double* x, double* hx, double* y, double* hy, double* z,
                              double* hz) {
    if (!cfg) return fail(TS_ERR_INVALID, "cfg is NULL");
    HostGrid g;
    std::string err;
    ts_status s = build_grid(*cfg, g, err);
    if (s != TS_OK) return fail(s, err);
    auto put = [](double* dst, const std::vector<double>& src) {
        if (dst) std::memcpy(dst, src.data(), src.size() * sizeof(double));
    };
    put(x, g.x); put(hx, g.hx); put(y, g.y); put(hy, g.hy); put(z, g.z); put(hz, g.hz);
    return TS_OK;
}

size_t ts_state_doubles(const ts_config* cfg, int32_t layout) {
    if (!cfg || cfg->n_dims < 1 || cfg->n_dims > 3) return 0;
    size_t nx = (size_t)cfg->nx, ny = cfg->n_dims > 1 ? (size_t)cfg->ny : 1, nz = cfg->n_dims > 2 ? (size_t)cfg->nz : 1;
    if (layout == TS_LAYOUT_WITH_GHOSTS) {
        nx += 2;
        if (cfg->n_dims > 1) ny += 2;
        if (cfg->n_dims > 2) nz += 2;
    }
    return nx * ny * nz * NV;
}

// splitmix64-style finaliser over a linear combination of the counters:
// the value depends only on (seed, i, j, k), never on traversal order.
double ts_hash_uniform(uint64_t seed, int64_t i, int64_t j, int64_t k) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ULL + (uint64_t)i * 0xBF58476D1CE4E5B9ULL +
                 (uint64_t)j * 0x94D049BB133111EBULL + (uint64_t)k * 0xD6E8FEB86659FD39ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
}

ts_status ts_fill_scenario(const ts_config* cfg, int32_t scenario, uint64_t seed, const double* prm,
                           int32_t n_params, double* values) {
    if (!cfg || !values) return fail(TS_ERR_INVALID, "NULL argument");
    static const int need[4] = {7, 5, 5, 16};
    if (scenario < 0 || scenario > 3) return fail(TS_ERR_INVALID, "unknown scenario");
    if (n_params < need[scenario] || !prm) return fail(TS_ERR_INVALID, "too few scenario parameters");
    HostGrid g;
    std::string err;
    ts_status s = build_grid(*cfg, g, err);
    if (s != TS_OK) return fail(s, err);
    const int nd = cfg->n_dims;
    const int nx = cfg->nx, ny = nd > 1 ? cfg->ny : 1, nz = nd > 2 ? cfg->nz : 1;
    const double gm1 = cfg->gamma - 1.0;
    const double pshift = cfg->eos == TS_EOS_STIFFENED_GAS ? cfg->gamma * cfg->p_inf : 0.0;
    auto energy = [&](double rho, double u, double v, double w, double p) {
        return (p + pshift) / gm1 + 0.5 * rho * (u * u + v * v + w * w);
    };
    size_t o = 0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i, o += NV) {
                const double xc = g.x[i + 1];
                const double yc = nd > 1 ? g.y[j + 1] : 0.0;
                const double zc = nd > 2 ? g.z[k + 1] : 0.0;
                double rho = 1.0, u = 0.0, v = 0.0, w = 0.0, p = 1.0;
                switch (scenario) {
                case TS_SCENARIO_SHOCK_TUBE:
                    if (xc > prm[0]) { rho = prm[4]; u = prm[5]; p = prm[6]; }
                    else { rho = prm[1]; u = prm[2]; p = prm[3]; }
                    break;
                case TS_SCENARIO_SHEAR_LAYER: {
                    const bool inner = std::fabs(yc - 0.5 * cfg->length[1]) < 0.25 * cfg->length[1];
                    rho = inner ? prm[0] : prm[1];
                    u = inner ? prm[2] : -prm[2];
                    p = prm[3];
                    v = prm[4] * (2.0 * ts_hash_uniform(seed, i, j, k) - 1.0);
                    break;
                }
                case TS_SCENARIO_BLAST: {
                    const double dx = xc - 0.5 * cfg->length[0];
                    const double dy = nd > 1 ? yc - 0.5 * cfg->length[1] : 0.0;
                    const double dz = nd > 2 ? zc - 0.5 * cfg->length[2] : 0.0;
                    rho = prm[0] * (1.0 + prm[4] * (2.0 * ts_hash_uniform(seed, i, j, k) - 1.0));
                    p = (dx * dx + dy * dy + dz * dz < prm[3] * prm[3]) ? prm[2] : prm[1];
                    break;
                }
                case TS_SCENARIO_QUADRANTS: {
                    const bool right = xc > 0.5 * cfg->length[0];
                    const bool top = nd > 1 ? yc > 0.5 * cfg->length[1] : true;
                    const int q = top ? (right ? 0 : 1) : (right ? 3 : 2);
                    rho = prm[4 * q + 0]; u = prm[4 * q + 1]; v = prm[4 * q + 2]; p = prm[4 * q + 3];
                    break;
                }
                }
                values[o + 0] = rho;
                values[o + 1] = rho * u;
                values[o + 2] = rho * v;
                values[o + 3] = rho * w;
                values[o + 4] = energy(rho, u, v, w, p);
            }
    return TS_OK;
}

}  // extern "C"
