// Solution files in the reference's formats (include/ts_fvm.h, ts_*_solution,
// ts_*_tecplot): the binary checkpoint of Kernel::SaveSolution /
// LoadSolution (src/kernel/kernel.h:992-1079) and the Tecplot text of
// Kernel::SaveSolutionToTecplot (kernel.h:1082-1413), for one domain (the
// reference's rank 0).  The text is produced with the same iostream
// formatting (std::scientific, default precision) and the same arithmetic
// order for the derived variables, so the files are byte-identical to the
// reference's for the same state.
//
// Asynchronous Tecplot writes snapshot the state to host memory on the
// calling thread and format/write it on a worker thread, so the device can
// continue stepping; ts_wait_writes (and ts_destroy) join them.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "ts_fvm.h"
#include "ts_internal.h"

namespace ts {
namespace {

struct Dims {
    int nd, nx, ny, nz;
};

Dims dims_of(const ts_config& c) {
    return Dims{c.n_dims, c.nx, c.n_dims > 1 ? c.ny : 1, c.n_dims > 2 ? c.nz : 1};
}

// The text of `count` lines, line n produced by put(buf, n) (which returns the
// line's length, at most 256 bytes), formatted by several threads into
// per-range buffers and written in order: the same bytes as the reference's
// line-by-line ofstream output (std::scientific with the default precision
// is printf's "%.6e"; std::endl and '\n' write the same byte).
template <class Put>
void write_lines(std::ofstream& ofs, long long count, Put put) {
    if (count <= 0) return;
    const long long per = 1 << 16;
    const int nt = (int)std::max<long long>(
        1, std::min<long long>((count + per - 1) / per, std::max(1u, std::thread::hardware_concurrency())));
    std::vector<std::string> parts(nt);
    auto work = [&](int t) {
        const long long b = count * t / nt, e = count * (t + 1) / nt;
        std::string& out = parts[t];
        out.reserve((size_t)(e - b) * 16);
        char buf[256];
        for (long long n = b; n < e; ++n) out.append(buf, (size_t)put(buf, n));
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& x : th) x.join();
    for (auto& p : parts) ofs.write(p.data(), (std::streamsize)p.size());
}

inline int put_e(char* buf, double x) { return std::snprintf(buf, 256, "%.6e\n", x); }

// Interior values are x fastest, then y, then z, 5 doubles per cell.
ts_status write_tecplot(const ts_config& c, const double* U, double time, double molar_mass, double gas_constant,
                        const std::string& path, std::string& err) {
    HostGrid g;
    ts_status s = build_grid(c, g, err);
    if (s != TS_OK) return s;
    const Dims d = dims_of(c);
    const double gamma = c.gamma;
    std::ofstream ofs(path, std::ios::binary);
    if (!ofs) { err = "cannot open " + path; return TS_ERR_INVALID; }
    ofs << std::scientific;
    const long long ncell = (long long)d.nx * d.ny * d.nz;
    auto cellv = [&](long long n, int v) { return U[n * 5 + v]; };
    if (d.nd == 1) {
        // kernel.h:1085-1149
        ofs << "VARIABLES = ";
        ofs << "\"" << "X" << "\" ";
        ofs << "\"" << "ro" << "\" ";
        ofs << "\"" << "u" << "\" ";
        ofs << "\"" << "v" << "\" ";
        ofs << "\"" << "w" << "\" ";
        ofs << "\"" << "P" << "\" ";
        ofs << "\"" << "e" << "\" ";
        ofs << '\n';
        write_lines(ofs, d.nx, [&](char* buf, long long i) {
            const double x = g.x[i + 1];
            const double ro = cellv(i, 0);
            const double u = cellv(i, 1) / ro;
            const double v = cellv(i, 2) / ro;
            const double w = cellv(i, 3) / ro;
            const double e = cellv(i, 4) / ro - 0.5 * (u * u + v * v + w * w);
            const double P = (gamma - 1.0) * ro * e;
            return std::snprintf(buf, 256, "%.6e %.6e %.6e %.6e %.6e %.6e %.6e \n", x, ro, u, v, w, P, e);
        });
        ofs.close();
        return ofs ? TS_OK : (err = "write failed: " + path, TS_ERR_INVALID);
    }
    const double cond = (gamma - 1.0) * molar_mass / gas_constant;
    std::vector<double> rho(ncell), u(ncell), v(ncell), w(ncell), P(ncell), e(ncell), T(ncell);
    if (d.nd == 2) {
        // kernel.h:1152-1262
        ofs << "VARIABLES = ";
        ofs << R"("X" )" << R"("Y" )" << R"("Rho" )" << R"("u" )" << R"("v" )" << R"("w" )" << R"("P" )"
            << R"("e")" << R"("T")";
        ofs << std::endl;
        ofs << R"(ZONE T=")" << time << R"(")";
        ofs << std::endl;
        ofs << "N=" << (d.nx + 1) * (d.ny + 1) << ", E=" << d.nx * d.ny << ", F=FEBLOCK, ET=QUADRILATERAL";
        ofs << std::endl;
        ofs << "VARLOCATION = (NODAL, NODAL";
        for (int k = 0; k < 6; ++k) ofs << ", CELLCENTERED";
        ofs << ", CELLCENTERED)";
        ofs << std::endl;
        const long long nxn = d.nx + 1, nyn = d.ny + 1;
        write_lines(ofs, nxn * nyn, [&](char* buf, long long n) {
            const long long i = n % nxn + 1;
            return put_e(buf, g.x[i] - 0.5 * g.hx[i]);
        });
        write_lines(ofs, nxn * nyn, [&](char* buf, long long n) {
            const long long j = n / nxn + 1;
            return put_e(buf, g.y[j] - 0.5 * g.hy[j]);
        });
        for (long long n = 0; n < ncell; ++n) {
            rho[n] = cellv(n, 0);
            u[n] = cellv(n, 1) / rho[n];
            v[n] = cellv(n, 2) / rho[n];
            w[n] = cellv(n, 3) / rho[n];
            e[n] = cellv(n, 4) / rho[n];
            e[n] = e[n] - 0.5 * (u[n] * u[n] + v[n] * v[n] + w[n] * w[n]);
            P[n] = (gamma - 1.0) * (rho[n] * e[n]);
            T[n] = cond * e[n];
        }
    } else {
        // kernel.h:1265-1406
        ofs << "VARIABLES = ";
        ofs << R"("X" )" << R"("Y" )" << R"("Z" )" << R"("Rho" )" << R"("u" )" << R"("v" )" << R"("w" )"
            << R"("P" )" << R"("e")" << R"("T")";
        ofs << std::endl;
        ofs << R"(ZONE T=")" << time << R"(")";
        ofs << std::endl;
        ofs << "N=" << (d.nx + 1) * (d.ny + 1) * (d.nz + 1) << ", E=" << d.nx * d.ny * d.nz
            << ", F=FEBLOCK, ET=BRICK";
        ofs << std::endl;
        ofs << "VARLOCATION = (NODAL, NODAL, NODAL";
        for (int k = 0; k < 6; ++k) ofs << ", CELLCENTERED";
        ofs << ", CELLCENTERED)";
        ofs << std::endl;
        const long long nxn = d.nx + 1, nyn = d.ny + 1, nzn = d.nz + 1;
        const long long nn = nxn * nyn * nzn;
        write_lines(ofs, nn, [&](char* buf, long long n) {
            const long long i = n % nxn + 1;
            return put_e(buf, g.x[i] - 0.5 * g.hx[i]);
        });
        write_lines(ofs, nn, [&](char* buf, long long n) {
            const long long j = (n / nxn) % nyn + 1;
            return put_e(buf, g.y[j] - 0.5 * g.hy[j]);
        });
        write_lines(ofs, nn, [&](char* buf, long long n) {
            const long long k = n / (nxn * nyn) + 1;
            return put_e(buf, g.z[k] - 0.5 * g.hz[k]);
        });
        for (long long n = 0; n < ncell; ++n) {
            rho[n] = cellv(n, 0);
            const double mx = cellv(n, 1), my = cellv(n, 2), mz = cellv(n, 3);
            const double kin = 0.5 * (mx * mx + my * my + mz * mz) / rho[n];
            u[n] = mx / rho[n];
            v[n] = my / rho[n];
            w[n] = mz / rho[n];
            e[n] = cellv(n, 4) - kin;
            P[n] = (gamma - 1.0) * (e[n]);
            e[n] /= rho[n];
            T[n] = cond * e[n];
        }
    }
    for (const std::vector<double>* a : {&rho, &u, &v, &w, &P, &e, &T})
        write_lines(ofs, ncell, [&](char* buf, long long n) { return put_e(buf, (*a)[n]); });
    if (d.nd == 2) {
        // cell (i, j): its four nodes, Tecplot node numbers starting at 1
        write_lines(ofs, (long long)d.nx * d.ny, [&](char* buf, long long n) {
            const int i = (int)(n % d.nx), j = (int)(n / d.nx);
            const int bl = (d.nx + 1) * j + 1 + i;
            const int br = bl + 1, ul = bl + (d.nx + 1), ur = ul + 1;
            return std::snprintf(buf, 256, "%d %d %d %d\n", bl, ul, ur, br);
        });
    } else {
        const int nxy = (d.nx + 1) * (d.ny + 1);
        write_lines(ofs, ncell, [&](char* buf, long long n) {
            const int i = (int)(n % d.nx), j = (int)((n / d.nx) % d.ny), k = (int)(n / ((long long)d.nx * d.ny));
            const int fbl = nxy * k + (d.nx + 1) * j + 1 + i;
            const int fbr = fbl + 1, ful = fbl + (d.nx + 1), fur = ful + 1;
            const int bbl = fbl + nxy, bbr = bbl + 1, bul = bbl + (d.nx + 1), bur = bul + 1;
            return std::snprintf(buf, 256, "%d %d %d %d %d %d %d %d\n", bbr, bur, bul, bbl, fbr, fur, ful, fbl);
        });
    }
    ofs.close();
    if (!ofs) { err = "write failed: " + path; return TS_ERR_INVALID; }
    return TS_OK;
}

// Pending asynchronous writes per handle.
struct Pending {
    std::vector<std::thread> threads;
    ts_status status = TS_OK;
    std::string error;
};
std::mutex g_io_mutex;
std::map<const ts_handle*, Pending> g_pending;

}  // namespace

void io_join_all(const ts_handle* h, ts_status* status, std::string* error) {
    std::vector<std::thread> ts;
    {
        std::lock_guard<std::mutex> lock(g_io_mutex);
        auto it = g_pending.find(h);
        if (it == g_pending.end()) return;
        ts.swap(it->second.threads);
    }
    for (auto& t : ts) t.join();
    std::lock_guard<std::mutex> lock(g_io_mutex);
    auto it = g_pending.find(h);
    if (it == g_pending.end()) return;
    if (status) *status = it->second.status;
    if (error) *error = it->second.error;
    g_pending.erase(it);
}

}  // namespace ts

using namespace ts;

extern "C" {

ts_status ts_write_solution_file(const ts_config* cfg, const double* values, double time, const char* path) {
    if (!cfg || !values || !path) return fail(TS_ERR_INVALID, "NULL argument");
    std::string err;
    if (validate_config(*cfg, err) != TS_OK) return fail(TS_ERR_INVALID, err);
    const Dims d = dims_of(*cfg);
    std::ofstream ofs(path, std::ios::binary | std::ios::out);
    if (!ofs) return fail(TS_ERR_INVALID, std::string("cannot open ") + path);
    const int32_t rank = 0;
    ofs.write(reinterpret_cast<const char*>(&time), sizeof time);
    ofs.write(reinterpret_cast<const char*>(&rank), sizeof rank);
    ofs.write(reinterpret_cast<const char*>(values), (std::streamsize)((size_t)d.nx * d.ny * d.nz * 5 * sizeof(double)));
    ofs.close();
    if (!ofs) return fail(TS_ERR_INVALID, std::string("write failed: ") + path);
    return TS_OK;
}

ts_status ts_read_solution_file(const ts_config* cfg, const char* path, double* values, double* time) {
    if (!cfg || !values || !path || !time) return fail(TS_ERR_INVALID, "NULL argument");
    std::string err;
    if (validate_config(*cfg, err) != TS_OK) return fail(TS_ERR_INVALID, err);
    const Dims d = dims_of(*cfg);
    const size_t n = (size_t)d.nx * d.ny * d.nz * 5;
    std::ifstream ifs(path, std::ios::binary | std::ios::in);
    if (!ifs) return fail(TS_ERR_INVALID, std::string("cannot open ") + path);
    int32_t rank = -1;
    ifs.read(reinterpret_cast<char*>(time), sizeof(double));
    ifs.read(reinterpret_cast<char*>(&rank), sizeof rank);
    if (!ifs) return fail(TS_ERR_INVALID, "truncated solution file");
    if (rank != 0)
        return fail(TS_ERR_UNSUPPORTED, "solution file's first block is rank " + std::to_string(rank) +
                                            "; one-domain files (rank 0) only");
    ifs.read(reinterpret_cast<char*>(values), (std::streamsize)(n * sizeof(double)));
    if (!ifs) return fail(TS_ERR_INVALID, "solution file shorter than the grid");
    return TS_OK;
}

ts_status ts_write_tecplot_file(const ts_config* cfg, const double* values, double time, double molar_mass,
                                double gas_constant, const char* path) {
    if (!cfg || !values || !path) return fail(TS_ERR_INVALID, "NULL argument");
    std::string err;
    if (validate_config(*cfg, err) != TS_OK) return fail(TS_ERR_INVALID, err);
    const ts_status s = write_tecplot(*cfg, values, time, molar_mass, gas_constant, path, err);
    return s == TS_OK ? TS_OK : fail(s, err);
}

ts_status ts_save_solution(ts_handle* h, const char* path) {
    if (!h || !path) return fail(TS_ERR_INVALID, "NULL argument");
    const ts_config& c = handle_config(h);
    std::vector<double> v(ts_state_doubles(&c, TS_LAYOUT_INTERIOR));
    ts_status s = ts_get_state(h, v.data(), TS_LAYOUT_INTERIOR);
    if (s != TS_OK) return s;
    ts_step_info info;
    if ((s = ts_get_step_info(h, &info)) != TS_OK) return s;
    return ts_write_solution_file(&c, v.data(), info.time, path);
}

ts_status ts_load_solution(ts_handle* h, const char* path) {
    if (!h || !path) return fail(TS_ERR_INVALID, "NULL argument");
    const ts_config& c = handle_config(h);
    std::vector<double> v(ts_state_doubles(&c, TS_LAYOUT_INTERIOR));
    double time = 0.0;
    ts_status s = ts_read_solution_file(&c, path, v.data(), &time);
    if (s != TS_OK) return s;
    if ((s = ts_set_state(h, v.data(), TS_LAYOUT_INTERIOR)) != TS_OK) return s;
    ts_step_info info;
    if ((s = ts_get_step_info(h, &info)) != TS_OK) return s;
    // LoadSolution keeps the iteration count and restarts the snapshot
    // schedule after the loaded time (kernel.h:1040-1041)
    info.time = time;
    if (c.save_solution_time > 0)
        info.next_solution_time = (int(time / c.save_solution_time) + 1) * c.save_solution_time;
    if (c.save_slice_time > 0) info.next_slice_time = (int(time / c.save_slice_time) + 1) * c.save_slice_time;
    return ts_set_step_info(h, &info);
}

ts_status ts_save_tecplot(ts_handle* h, const char* path, double molar_mass, double gas_constant, int32_t async) {
    if (!h || !path) return fail(TS_ERR_INVALID, "NULL argument");
    const ts_config c = handle_config(h);
    auto v = std::make_shared<std::vector<double>>(ts_state_doubles(&c, TS_LAYOUT_INTERIOR));
    ts_status s = ts_get_state(h, v->data(), TS_LAYOUT_INTERIOR);
    if (s != TS_OK) return s;
    ts_step_info info;
    if ((s = ts_get_step_info(h, &info)) != TS_OK) return s;
    if (!async) return ts_write_tecplot_file(&c, v->data(), info.time, molar_mass, gas_constant, path);
    const std::string p(path);
    const double time = info.time;
    std::lock_guard<std::mutex> lock(g_io_mutex);
    Pending& pend = g_pending[h];
    pend.threads.emplace_back([h, c, v, time, molar_mass, gas_constant, p] {
        std::string err;
        const ts_status st = write_tecplot(c, v->data(), time, molar_mass, gas_constant, p, err);
        if (st != TS_OK) {
            std::lock_guard<std::mutex> lk(g_io_mutex);
            Pending& q = g_pending[h];
            if (q.status == TS_OK) { q.status = st; q.error = err; }
        }
    });
    return TS_OK;
}

ts_status ts_wait_writes(ts_handle* h) {
    if (!h) return fail(TS_ERR_INVALID, "NULL handle");
    ts_status st = TS_OK;
    std::string err;
    io_join_all(h, &st, &err);
    return st == TS_OK ? TS_OK : fail(st, err);
}

}  // extern "C"
