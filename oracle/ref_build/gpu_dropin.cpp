// Build check of the GPU drop-in (include/ts_kernel.hpp) against the
// reference's own headers, written for this project and compiled into the
// git-ignored oracle/_ref/ directory by `make -C oracle/ref_build dropin`.
//
// Two problems are set up exactly as the reference's experiment drivers do
// (a KernelConfiguration, Init, SetInitialConditions, Run; cf.
// src/Tests/1DTests/ToroTests.h:395-449 and src/Tests/2DTests/BlasiusFlow.h:
// 70-140): a 1D Sod tube and a 2D channel with a plate on the bottom side
// (a position-dependent side: DomainBCinfo::isComplex with getMarker).
//
//   gpu_dropin --config   print the ts_config GpuExplicitRungeKuttaFVM
//                         builds for each problem (no GPU needed)
//   gpu_dropin            run each problem with the reference's CPU kernel
//                         (CreateKernel) and with CreateGpuKernel (FP64 and
//                         mixed precision) and print the largest relative
//                         difference of the final values
#include "Methods/ExplicitRungeKuttaFVM.h"
#include "ts_kernel.hpp"

#include <cstdio>
#include <cstring>

namespace {

struct Problem {
    const char* name;
    KernelConfiguration conf;
    std::function<std::vector<double>(const Vector&)> ic;
};

std::vector<double> conserved(double g, double rho, double u, double v, double p) {
    return {rho, rho * u, rho * v, 0.0, p / (g - 1.0) + 0.5 * rho * (u * u + v * v)};
}

Problem sod() {
    Problem pr;
    pr.name = "sod1d";
    KernelConfiguration& c = pr.conf;
    c.nDims = 1;
    c.nX = 200;
    c.isPeriodicX = false;
    c.LX = 1.0;
    c.Gamma = 1.4;
    c.MyConditions[1] = BoundaryConditionConfiguration(BoundaryConditionType::Natural);
    c.xLeftBoundary.SetMarker(1);
    c.xRightBoundary.SetMarker(1);
    c.methodConfiguration.CFL = 0.5;
    c.methodConfiguration.RungeKuttaOrder = 1;
    c.methodConfiguration.Eps = 0.0;
    c.methodConfiguration.RiemannProblemSolver = RPSolver::RoePikeSolver;
    c.methodConfiguration.ReconstructionType = Reconstruction::PiecewiseConstant;
    c.DummyLayerSize = 1;
    c.MaxTime = 0.2;
    c.MaxIteration = 1000000;
    c.SaveSolutionTime = 0.05;
    c.SaveHistoryFileIters = 1 << 30;
    c.ResidualOutputIters = 0;
    const double g = c.Gamma;
    pr.ic = [g](const Vector& r) {
        return r.x < 0.5 ? conserved(g, 1.0, 0.0, 0.0, 1.0) : conserved(g, 0.125, 0.0, 0.0, 0.1);
    };
    return pr;
}

Problem plate() {
    Problem pr;
    pr.name = "plate2d";
    KernelConfiguration& c = pr.conf;
    c.nDims = 2;
    c.nX = 64;
    c.nY = 32;
    c.isPeriodicX = false;
    c.isPeriodicY = false;
    c.LX = 1.0;
    c.LY = 0.5;
    c.Gamma = 1.4;
    BoundaryConditionConfiguration inlet(BoundaryConditionType::SubsonicInlet);
    inlet.Density = 1.0;
    inlet.Pstatic = 1.0 / 1.4;
    inlet.Velocity = Vector(0.5, 0.0, 0.0);
    c.MyConditions[1] = inlet;
    c.MyConditions[2] = BoundaryConditionConfiguration(BoundaryConditionType::Natural);
    c.MyConditions[3] = BoundaryConditionConfiguration(BoundaryConditionType::Wall);
    c.MyConditions[4] = BoundaryConditionConfiguration(BoundaryConditionType::Symmetry);
    c.xLeftBoundary.SetMarker(1);
    c.xRightBoundary.SetMarker(2);
    c.yRightBoundary.SetMarker(2);
    c.yLeftBoundary.isComplex = true;
    c.yLeftBoundary.getMarker = [](Vector r) { return r.x < 0.3 ? 4 : 3; };
    c.methodConfiguration.CFL = 0.45;
    c.methodConfiguration.RungeKuttaOrder = 1;
    c.methodConfiguration.Eps = 0.05;
    c.methodConfiguration.RiemannProblemSolver = RPSolver::RoePikeSolver;
    c.methodConfiguration.ReconstructionType = Reconstruction::Linear2psLim;
    c.methodConfiguration.GeneralLimitter = LimiterType::BarsJespersen;
    c.DummyLayerSize = 1;
    c.MaxTime = 1e9;
    c.MaxIteration = 200;
    c.SaveHistoryFileIters = 1 << 30;
    c.ResidualOutputIters = 0;
    const double g = c.Gamma;
    pr.ic = [g](const Vector& r) { return conserved(g, 1.0, 0.5, 0.0, 1.0 / 1.4); };
    return pr;
}

}  // namespace

int main(int argc, char* argv[]) {
    const bool config_only = argc > 1 && std::strcmp(argv[1], "--config") == 0;
    Problem problems[2] = {sod(), plate()};
    int rc = 0;
    for (Problem& pr : problems) {
        std::unique_ptr<Kernel> cpu = CreateKernel(pr.conf, argc, argv);
        cpu->Init(pr.conf);
        cpu->SetInitialConditions(pr.ic);
        if (config_only) {
            std::vector<ts_block_node> blocks[3];
            std::vector<uint8_t> marks[6];
            const ts_config c =
                GpuExplicitRungeKuttaFVM::MakeConfig(pr.conf, cpu->grid, TS_PRECISION_MIXED, 0, blocks, marks);
            std::printf("%s n_dims %d nx %d ny %d periodic %d %d recon %d limiter %d solver %d cfl %.17g eps %.17g "
                        "max_iter %d max_time %.17g save_solution_time %.17g precision %d residual_norms %d\n",
                        pr.name, c.n_dims, c.nx, c.ny, c.periodic[0], c.periodic[1], c.reconstruction, c.limiter,
                        c.riemann_solver, c.cfl, c.eps, c.max_iteration, c.max_time, c.save_solution_time,
                        c.precision, c.residual_norms);
            for (int s = 0; s < 2 * c.n_dims; ++s) {
                std::printf("%s side %d type %d density %.17g velocity %.17g %.17g %.17g pstatic %.17g markers",
                            pr.name, s, c.bc[s].type, c.bc[s].density, c.bc[s].velocity[0], c.bc[s].velocity[1],
                            c.bc[s].velocity[2], c.bc[s].pstatic);
                if (c.bc_marker[s])
                    for (int f = 0; f < (s < 2 ? c.ny : c.nx); ++f) std::printf(" %d", c.bc_marker[s][f]);
                std::printf("\n");
            }
            for (int k = 0; k < c.n_bc_kinds; ++k) std::printf("%s kind %d type %d\n", pr.name, k, c.bc_kinds[k].type);
            continue;
        }
        cpu->Run();
        for (int precision : {TS_PRECISION_FP64, TS_PRECISION_MIXED}) {
            std::unique_ptr<Kernel> gpu = CreateGpuKernel(pr.conf, argc, argv, precision);
            try {
                gpu->Init(pr.conf);
                gpu->SetInitialConditions(pr.ic);
                gpu->Run();
            } catch (const std::exception& e) {
                std::printf("%s precision %d: %s\n", pr.name, precision, e.what());
                rc = 3;
                break;
            }
            double dmax = 0.0, vmax = 0.0;
            for (size_t i = 0; i < cpu->values.size(); ++i) {
                dmax = std::max(dmax, std::fabs(gpu->values[i] - cpu->values[i]));
                vmax = std::max(vmax, std::fabs(cpu->values[i]));
            }
            std::printf("%s precision %d iterations %d/%d time %.17g/%.17g max relative difference %.3e\n", pr.name,
                        precision, gpu->stepInfo.Iteration, cpu->stepInfo.Iteration, gpu->stepInfo.Time,
                        cpu->stepInfo.Time, dmax / vmax);
            if (gpu->stepInfo.Iteration != cpu->stepInfo.Iteration) rc = 1;
            if (precision == TS_PRECISION_FP64 && dmax != 0.0) rc = 1;
            if (precision == TS_PRECISION_MIXED && dmax / vmax > 1e-4) rc = 1;
        }
    }
    return rc;
}
