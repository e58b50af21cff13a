// Test-oracle driver around the reference solver's own CPU path
// (ExplicitRungeKuttaFVM<R>, src/Methods/ExplicitRungeKuttaFVM.h:15-1493).
// Written for this project: it builds a KernelConfiguration from a small
// text file, loads an initial state, calls the reference's Init/Run exactly as
// its experiment drivers do (e.g. src/Tests/1DTests/ToroTests.h:395-449), and
// dumps the final state, step info and grid to a binary file.  It is only
// ever compiled into the git-ignored oracle/_ref/ directory.
//
// Config file: one "key value..." per line ('#' starts a comment).
//   ndims nx ny nz periodic_x periodic_y periodic_z lx ly lz gamma
//   recon (0 PWC, 1 Linear2PointsStencil, 2 ENO2, 3 Linear2psLim)
//   limiter (0 BarsJespersen, 1 Venkatakrishnan)  solver (0 Godunov, 1 Roe)
//   eps cfl rk_order max_iter max_time save_solution_time save_slice_time
//   bc_xl|bc_xr|bc_yl|bc_yr|bc_zl|bc_zr  type [density vx vy vz pstatic]
//       (type = BoundaryConditionType value, BoundaryConditionConfiguration.h:12-19)
//   bc_kind m type [density vx vy vz pstatic]   (extra MyConditions entry, marker 100+m)
//   bc_split side axis pos m_lo m_hi   (side 0..5 = x-,x+,y-,y+,z-,z+ made complex:
//       DomainBCinfo::isComplex with getMarker(r) = r[axis] < pos ? 100+m_lo : 100+m_hi,
//       BoundaryConditionConfiguration.h:43-66, as src/Tests/2DTests/BlasiusFlow.h:115-120)
//   blocks_x|blocks_y|blocks_z  n  pos q ncells  pos q ncells ...
//   ic_file path   (interior cells, x fastest then y then z, 5 doubles each)
//   out_file path
//   toro N        (optional: Toro test N initial data by the reference's own
//                  cell-averaged quadrature, ToroTests.h:426-446, plus the
//                  exact solution and error norms, ToroTests.h:451-457)
//   steps N       (optional: call IterationStep N times instead of Run)
//   load_solution path   (optional: Kernel::LoadSolution before stepping)
//   save_solution path   (optional: Kernel::SaveSolution after stepping)
//   save_tecplot path    (optional: Kernel::SaveSolutionToTecplot after stepping)
//   molar_mass x, gas_constant x   (KernelConfiguration MolarMass, UniversalGasConstant)
//   external_force sx sy sz        (IsExternalForceRequared with Sigma)
//   uniform_acceleration gx gy gz  (IsUnifromAccelerationRequared with UniformAcceleration)
//   viscous 0|1, viscosity mu      (IsViscousFlow, Viscosity)
#include "Methods/ExplicitRungeKuttaFVM.h"
#include "Tests/1DTests/ToroTests.h"

#include <cstdint>

namespace {

struct DriverConfig {
    KernelConfiguration conf;
    std::string ic_file, out_file;
    std::string load_solution, save_solution, save_tecplot;
    int toro = 0;
    int steps = -1;
    std::vector<BlockNode> blocks[3];
    bool has_blocks[3] = {false, false, false};
};

std::vector<std::string> split(const std::string& s) {
    std::istringstream is(s);
    std::vector<std::string> out;
    std::string w;
    while (is >> w) out.push_back(w);
    return out;
}

void set_bc(KernelConfiguration& conf, DomainBCinfo& side, int marker, const std::vector<std::string>& w) {
    BoundaryConditionConfiguration bc((BoundaryConditionType)std::stoi(w[1]));
    bc.Density = w.size() > 2 ? std::stod(w[2]) : 0.0;
    bc.Velocity = Vector(w.size() > 3 ? std::stod(w[3]) : 0.0, w.size() > 4 ? std::stod(w[4]) : 0.0,
                         w.size() > 5 ? std::stod(w[5]) : 0.0);
    bc.Pstatic = w.size() > 6 ? std::stod(w[6]) : 0.0;
    conf.MyConditions[marker] = bc;
    side.SetMarker(marker);
}

void set_kind(KernelConfiguration& conf, const std::vector<std::string>& w) {
    BoundaryConditionConfiguration bc((BoundaryConditionType)std::stoi(w[2]));
    bc.Density = w.size() > 3 ? std::stod(w[3]) : 0.0;
    bc.Velocity = Vector(w.size() > 4 ? std::stod(w[4]) : 0.0, w.size() > 5 ? std::stod(w[5]) : 0.0,
                         w.size() > 6 ? std::stod(w[6]) : 0.0);
    bc.Pstatic = w.size() > 7 ? std::stod(w[7]) : 0.0;
    conf.MyConditions[100 + std::stoi(w[1])] = bc;
}

void set_split(KernelConfiguration& conf, const std::vector<std::string>& w) {
    DomainBCinfo* sides[6] = {&conf.xLeftBoundary, &conf.xRightBoundary, &conf.yLeftBoundary,
                              &conf.yRightBoundary, &conf.zLeftBoundary, &conf.zRightBoundary};
    DomainBCinfo& side = *sides[std::stoi(w[1])];
    const int axis = std::stoi(w[2]);
    const double pos = std::stod(w[3]);
    const int lo = 100 + std::stoi(w[4]), hi = 100 + std::stoi(w[5]);
    side.isComplex = true;
    side.getMarker = [axis, pos, lo, hi](const Vector r) {
        const double c = axis == 0 ? r.x : (axis == 1 ? r.y : r.z);
        return c < pos ? lo : hi;
    };
}

DriverConfig parse(const char* path) {
    DriverConfig d;
    KernelConfiguration& c = d.conf;
    c.DummyLayerSize = 1;
    c.SaveHistoryFileIters = 1 << 30;
    c.ResidualOutputIters = 0;
    std::ifstream in(path);
    if (!in) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    std::string line;
    while (std::getline(in, line)) {
        auto h = line.find('#');
        if (h != std::string::npos) line = line.substr(0, h);
        auto w = split(line);
        if (w.empty()) continue;
        const std::string& k = w[0];
        auto D = [&](int i) { return std::stod(w[i]); };
        auto I = [&](int i) { return std::stoi(w[i]); };
        if (k == "ndims") c.nDims = I(1);
        else if (k == "nx") c.nX = I(1);
        else if (k == "ny") c.nY = I(1);
        else if (k == "nz") c.nZ = I(1);
        else if (k == "periodic_x") c.isPeriodicX = I(1) != 0;
        else if (k == "periodic_y") c.isPeriodicY = I(1) != 0;
        else if (k == "periodic_z") c.isPeriodicZ = I(1) != 0;
        else if (k == "lx") c.LX = D(1);
        else if (k == "ly") c.LY = D(1);
        else if (k == "lz") c.LZ = D(1);
        else if (k == "gamma") c.Gamma = D(1);
        else if (k == "recon") c.methodConfiguration.ReconstructionType = (Reconstruction)I(1);
        else if (k == "limiter") c.methodConfiguration.GeneralLimitter = (LimiterType)I(1);
        else if (k == "solver") c.methodConfiguration.RiemannProblemSolver = (RPSolver)I(1);
        else if (k == "eps") c.methodConfiguration.Eps = D(1);
        else if (k == "cfl") c.methodConfiguration.CFL = D(1);
        else if (k == "rk_order") c.methodConfiguration.RungeKuttaOrder = I(1);
        else if (k == "max_iter") c.MaxIteration = I(1);
        else if (k == "max_time") c.MaxTime = D(1);
        else if (k == "save_solution_time") c.SaveSolutionTime = D(1);
        else if (k == "save_slice_time") c.SaveSliceTime = D(1);
        else if (k == "bc_xl") set_bc(c, c.xLeftBoundary, 1, w);
        else if (k == "bc_xr") set_bc(c, c.xRightBoundary, 2, w);
        else if (k == "bc_yl") set_bc(c, c.yLeftBoundary, 3, w);
        else if (k == "bc_yr") set_bc(c, c.yRightBoundary, 4, w);
        else if (k == "bc_zl") set_bc(c, c.zLeftBoundary, 5, w);
        else if (k == "bc_zr") set_bc(c, c.zRightBoundary, 6, w);
        else if (k == "bc_kind") set_kind(c, w);
        else if (k == "bc_split") set_split(c, w);
        else if (k == "blocks_x" || k == "blocks_y" || k == "blocks_z") {
            int a = k[7] - 'x';
            int n = I(1);
            d.blocks[a].clear();
            for (int b = 0; b < n; ++b) {
                BlockNode node(D(2 + 3 * b));
                node.q_com = D(3 + 3 * b);
                node.N_cells = I(4 + 3 * b);
                d.blocks[a].push_back(node);
            }
            d.has_blocks[a] = true;
        }
        else if (k == "ic_file") d.ic_file = w[1];
        else if (k == "out_file") d.out_file = w[1];
        else if (k == "toro") d.toro = I(1);
        else if (k == "steps") d.steps = I(1);
        else if (k == "load_solution") d.load_solution = w[1];
        else if (k == "save_solution") d.save_solution = w[1];
        else if (k == "save_tecplot") d.save_tecplot = w[1];
        else if (k == "external_force") {
            c.IsExternalForceRequared = true;
            c.Sigma = Vector(D(1), D(2), D(3));
        }
        else if (k == "uniform_acceleration") {
            c.IsUnifromAccelerationRequared = true;
            c.UniformAcceleration = Vector(D(1), D(2), D(3));
        }
        else if (k == "viscous") c.IsViscousFlow = I(1) != 0;
        else if (k == "viscosity") c.Viscosity = D(1);
        else if (k == "molar_mass") c.MolarMass = D(1);
        else if (k == "gas_constant") c.UniversalGasConstant = D(1);
        else { std::fprintf(stderr, "unknown key %s\n", k.c_str()); std::exit(2); }
    }
    if (d.has_blocks[0]) c.CompressionX = d.blocks[0];
    if (d.has_blocks[1]) c.CompressionY = d.blocks[1];
    if (d.has_blocks[2]) c.CompressionZ = d.blocks[2];
    return d;
}

std::unique_ptr<Kernel> make_kernel(KernelConfiguration& conf, int argc, char** argv) {
    // Same template choice as CreateKernel (ExplicitRungeKuttaFVM.h:1496-1513),
    // plus Linear2PointsStencil, which CreateKernel leaves unhandled.
    if (conf.methodConfiguration.ReconstructionType == Reconstruction::Linear2PointsStencil)
        return std::unique_ptr<Kernel>(new ExplicitRungeKuttaFVM<Linear2PointsStencil>(&argc, &argv));
    return CreateKernel(conf, argc, argv);
}

void write_vec(std::ofstream& o, const std::valarray<double>& v) {
    int64_t n = (int64_t)v.size();
    o.write(reinterpret_cast<const char*>(&n), sizeof n);
    if (n) o.write(reinterpret_cast<const char*>(&v[0]), n * sizeof(double));
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) { std::fprintf(stderr, "usage: ref_run config.txt\n"); return 2; }
    DriverConfig d = parse(argv[1]);
    KernelConfiguration& conf = d.conf;

    ToroTests::ShockTubeParameters toro_params;
    if (d.toro > 0) {
        // Same settings as ToroTests::RunSingleExperiment (ToroTests.h:400-405),
        // keeping the resolution, reconstruction and solver from the file.
        KernelConfiguration t = ToroTests::DefaultSettings();
        toro_params = ToroTests::DefaultState(d.toro);
        t.nX = conf.nX;
        t.MaxTime = toro_params.t_res;
        t.methodConfiguration.ReconstructionType = conf.methodConfiguration.ReconstructionType;
        t.methodConfiguration.GeneralLimitter = conf.methodConfiguration.GeneralLimitter;
        t.methodConfiguration.RiemannProblemSolver = conf.methodConfiguration.RiemannProblemSolver;
        t.SaveHistoryFileIters = conf.SaveHistoryFileIters;
        t.ResidualOutputIters = 0;
        conf = t;
    }

    std::unique_ptr<Kernel> kernel = make_kernel(conf, argc, argv);
    if (!kernel) { std::fprintf(stderr, "unsupported reconstruction\n"); return 3; }
    kernel->Init(conf);
    Grid& g = kernel->grid;

    if (d.toro > 0) {
        NumericQuadrature integ(3, 1);
        auto p = toro_params;
        auto initD = [p](Vector r) {
            double pr = p.PL, u = p.uL, ro = p.roL;
            if (r.x > p.x0) { pr = p.PR; u = p.uR; ro = p.roR; }
            std::vector<double> res(5);
            res[0] = ro; res[1] = ro * u; res[2] = 0; res[3] = 0;
            res[4] = pr / TestsUtility::gamma1 + 0.5 * ro * u * u;
            return res;
        };
        kernel->SetInitialConditions(initD, integ);
    } else {
        std::ifstream ic(d.ic_file, std::ios::binary);
        if (!ic) { std::fprintf(stderr, "cannot open ic %s\n", d.ic_file.c_str()); return 2; }
        for (int k = g.kMin; k <= g.kMax; ++k)
            for (int j = g.jMin; j <= g.jMax; ++j)
                for (int i = g.iMin; i <= g.iMax; ++i)
                    ic.read(reinterpret_cast<char*>(kernel->getCellValues(i, j, k)), 5 * sizeof(double));
        if (!ic) { std::fprintf(stderr, "short ic file\n"); return 2; }
    }
    if (!d.load_solution.empty()) kernel->LoadSolution(d.load_solution);
    std::valarray<double> initial = kernel->values;

    auto t0 = std::chrono::steady_clock::now();
    if (d.steps >= 0) {
        for (int s = 0; s < d.steps; ++s) kernel->IterationStep();
    } else {
        kernel->Run();
    }
    auto t1 = std::chrono::steady_clock::now();
    double seconds = std::chrono::duration<double>(t1 - t0).count();
    if (!d.save_solution.empty()) kernel->SaveSolution(d.save_solution);
    if (!d.save_tecplot.empty()) kernel->SaveSolutionToTecplot(d.save_tecplot);

    std::ofstream o(d.out_file, std::ios::binary);
    const int32_t hdr[8] = {0x54534631, kernel->nDims, g.nlocalXAll, g.nlocalYAll, g.nlocalZAll,
                            kernel->stepInfo.Iteration, d.toro, 0};
    o.write(reinterpret_cast<const char*>(hdr), sizeof hdr);
    const double sc[4] = {kernel->stepInfo.Time, kernel->stepInfo.TimeStep, seconds, 0.0};
    o.write(reinterpret_cast<const char*>(sc), sizeof sc);
    write_vec(o, g.CoordinateX); write_vec(o, g.hx);
    write_vec(o, g.CoordinateY); write_vec(o, g.hy);
    write_vec(o, g.CoordinateZ); write_vec(o, g.hz);
    write_vec(o, g.volumes);
    write_vec(o, initial);
    write_vec(o, kernel->values);
    std::valarray<double> resid(kernel->stepInfo.Residual.data(), kernel->stepInfo.Residual.size());
    write_vec(o, resid);
    if (d.toro > 0) {
        TestsUtility::exact_solution =
            ToroTests::ComputeExactSolution(d.toro, toro_params, g, kernel->stepInfo.Time);
        std::valarray<double> inner(&(kernel->values[TestsUtility::nVar * g.dummyCellLayersX]),
                                    g.nlocalX * kernel->nVariables);
        std::vector<double> L2 = TestsUtility::ComputeL2Error(inner, g, *(kernel->pManager), conf.nX);
        std::vector<double> L1 = TestsUtility::ComputeL1Error(inner, g, *(kernel->pManager), conf.nX);
        std::valarray<double> errs(10);
        for (int v = 0; v < 5; ++v) { errs[v] = L2[v]; errs[5 + v] = L1[v]; }
        write_vec(o, TestsUtility::exact_solution);
        write_vec(o, errs);
    }
    o.close();
    std::printf("iterations %d time %.17g dt %.17g seconds %.6f\n", kernel->stepInfo.Iteration,
                kernel->stepInfo.Time, kernel->stepInfo.TimeStep, seconds);
    return 0;
}
