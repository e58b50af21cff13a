/*
 * ts_kernel.hpp -- the reference's Kernel plugin, run on the GPU.
 *
 * GpuExplicitRungeKuttaFVM is a Kernel (src/kernel/kernel.h:42-45: the
 * abstract IterationStep / InitializeMethod pair) whose step is the explicit
 * FVM step of ExplicitRungeKuttaFVM<R> (src/Methods/ExplicitRungeKuttaFVM.h:
 * 1440-1491) executed by libtsfvm.so through the C ABI in ts_fvm.h.
 * CreateGpuKernel has the signature of the reference's factory CreateKernel
 * (ExplicitRungeKuttaFVM.h:1496-1513), so a driver that builds a
 * KernelConfiguration, calls Init, SetInitialConditions and Run (e.g.
 * src/Tests/1DTests/ToroTests.h:395-449) runs unchanged on the GPU when it
 * takes its kernel from CreateGpuKernel instead of CreateKernel.
 *
 * Include it after the reference's "kernel/kernel.h" (it needs Kernel,
 * KernelConfiguration, Grid and the BC configuration types) and link
 * libtsfvm.so.  Header-only.
 *
 * Mirror of Kernel::values.  The state lives on the device.  The host copy
 * is uploaded before the first step (so SetInitialConditions or LoadSolution
 * called after Init need nothing else), and downloaded only after a step
 * whose results the Run loop reads (kernel.h:1700-1846): a sensor record, a
 * snapshot by iterations or by time (Tecplot, slices, binary), or the end of
 * the run (MaxIteration / MaxTime) -- not every step.
 * SaveSolutionToTecplot downloads first as well.  A caller that writes
 * `values` itself between steps calls SyncToDevice(); one that reads them
 * between steps outside those points calls SyncFromDevice().
 *
 * Step information: Time, Iteration, TimeStep and Residual come from the
 * device after every step; the snapshot times that Run advances on the host
 * are passed to the device before the next step, so dt is clipped to them as
 * in the reference (ExplicitRungeKuttaFVM.h:1433-1434).  With
 * TS_PRECISION_MIXED the residual norms are formed too (ts_config.
 * residual_norms), so history.dat is the same file as with the FP64 path.
 *
 * Boundary conditions: each side's marker selects its entry of
 * KernelConfiguration::MyConditions; a side with isComplex set has its
 * getMarker evaluated at every boundary face's centre (the point
 * ComputeResidual passes, ExplicitRungeKuttaFVM.h:1193-1209) and the
 * resulting per-face kinds go to ts_config.bc_kinds / bc_marker.
 *
 * Errors: a failing C ABI call throws std::runtime_error with
 * ts_last_error() (the reference signals errors with exceptions,
 * IReconstruction.h:39).  The reference's CreateKernel returns null for a
 * reconstruction it has no kernel for; CreateGpuKernel does the same for
 * configurations libtsfvm.so does not build.
 */
#ifndef TS_KERNEL_HPP
#define TS_KERNEL_HPP

#include <cmath>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ts_fvm.h"

class GpuExplicitRungeKuttaFVM : public Kernel {
public:
    // precision: TS_PRECISION_MIXED (FP32 flux, FP64 state: the fast path) or
    // TS_PRECISION_FP64 (bit for bit with the reference).  Configurations the
    // mixed path does not take (viscous flow, the exact Godunov solver) run
    // in FP64 either way.
    GpuExplicitRungeKuttaFVM(int* argc, char** argv[], int precision = TS_PRECISION_MIXED, int device = 0)
        : Kernel(argc, argv), precision_(precision), device_(device) {}
    // Kernel has no virtual destructor, so an object deleted through a Kernel
    // pointer (the unique_ptr<Kernel> CreateKernel's signature returns) does
    // not run this one: call Release() before, or the device memory is held
    // until the process exits.
    ~GpuExplicitRungeKuttaFVM() { Release(); }
    void Release() {
        if (h_) ts_destroy(h_);
        h_ = nullptr;
    }

    // The ts_config of a KernelConfiguration on this kernel's grid (Init has
    // run).  `marks` receives the per-face marker arrays it points to.
    static ts_config MakeConfig(KernelConfiguration& c, const Grid& grid, int precision, int device,
                                std::vector<ts_block_node> (&blocks)[3], std::vector<uint8_t> (&marks)[6]) {
        ts_config cfg{};
        cfg.abi_version = TS_FVM_ABI_VERSION;
        cfg.n_dims = c.nDims;
        cfg.nx = c.nX;
        cfg.ny = c.nY;
        cfg.nz = c.nZ;
        cfg.periodic[0] = c.isPeriodicX;
        cfg.periodic[1] = c.isPeriodicY;
        cfg.periodic[2] = c.isPeriodicZ;
        cfg.length[0] = c.LX;
        cfg.length[1] = c.LY;
        cfg.length[2] = c.LZ;
        const std::vector<BlockNode>* comp[3] = {&c.CompressionX, &c.CompressionY, &c.CompressionZ};
        for (int a = 0; a < 3; ++a) {
            blocks[a].clear();
            // Grid::InitGlobal (grid.h:164-170) has appended the closing
            // border node (no cells) and given a uniform axis's single node
            // its cell count; one node with q = 1 is a uniform axis
            if (a < c.nDims)
                for (const BlockNode& b : *comp[a])
                    if (b.N_cells >= 1) blocks[a].push_back(ts_block_node{b.pos, b.q_com, b.N_cells, 0});
            if (blocks[a].size() == 1 && blocks[a][0].q_com == 1.0) blocks[a].clear();
            cfg.n_blocks[a] = (int32_t)blocks[a].size();
            cfg.blocks[a] = blocks[a].empty() ? nullptr : blocks[a].data();
        }
        cfg.gamma = c.Gamma;
        cfg.eos = TS_EOS_IDEAL_GAS;
        const MethodConfiguration& m = c.methodConfiguration;
        cfg.reconstruction = (int32_t)m.ReconstructionType;
        cfg.riemann_solver = (int32_t)m.RiemannProblemSolver;
        cfg.limiter = (int32_t)m.GeneralLimitter;
        cfg.rk_order = m.RungeKuttaOrder;
        cfg.cfl = m.CFL;
        cfg.eps = m.Eps;
        cfg.max_iteration = c.MaxIteration;
        cfg.max_time = c.MaxTime;
        cfg.save_solution_time = c.SaveSolutionTime;
        cfg.save_slice_time = c.SaveSliceTime;
        cfg.external_force = c.IsExternalForceRequared;
        cfg.uniform_acceleration = c.IsUnifromAccelerationRequared;
        cfg.sigma[0] = c.Sigma.x;
        cfg.sigma[1] = c.Sigma.y;
        cfg.sigma[2] = c.Sigma.z;
        cfg.acceleration[0] = c.UniformAcceleration.x;
        cfg.acceleration[1] = c.UniformAcceleration.y;
        cfg.acceleration[2] = c.UniformAcceleration.z;
        cfg.viscous = c.IsViscousFlow;
        cfg.viscosity = c.Viscosity;
        const bool fp64_only = c.IsViscousFlow || c.Viscosity != 0.0 || m.RiemannProblemSolver == RPSolver::GodunovSolver;
        cfg.precision = fp64_only ? TS_PRECISION_FP64 : precision;
        cfg.residual_norms = cfg.precision == TS_PRECISION_MIXED;
        cfg.device = device;

        // boundary conditions (Kernel::InitBoundaryConditions, kernel.h:284-316)
        DomainBCinfo* sides[6] = {&c.xLeftBoundary, &c.xRightBoundary, &c.yLeftBoundary,
                                  &c.yRightBoundary, &c.zLeftBoundary, &c.zRightBoundary};
        std::map<int, int> kind_of_marker;  // MyConditions marker -> bc_kinds index
        for (int s = 0; s < 6; ++s) {
            marks[s].clear();
            cfg.bc_marker[s] = nullptr;
            const int a = s / 2;
            cfg.bc[s].type = TS_BC_NATURAL;
            if (a >= c.nDims || cfg.periodic[a]) continue;
            if (!sides[s]->isComplex) {
                cfg.bc[s] = to_bc(c.MyConditions.at(sides[s]->GetMarker()));
                continue;
            }
            // getMarker at each boundary face's centre, faces numbered by
            // the tangential interior cells, lower axis fastest
            const int n[3] = {grid.nX, c.nDims > 1 ? grid.nY : 1, c.nDims > 2 ? grid.nZ : 1};
            const int off[3] = {grid.iMin, c.nDims > 1 ? grid.jMin : 0, c.nDims > 2 ? grid.kMin : 0};
            const int t0 = a == 0 ? 1 : 0, t1 = a == 2 ? 1 : 2;
            const int hi = s % 2;
            for (int q = 0; q < n[t1]; ++q)
                for (int p = 0; p < n[t0]; ++p) {
                    int idx[3];
                    idx[t0] = p + off[t0];
                    idx[t1] = q + off[t1];
                    idx[a] = hi ? off[a] + n[a] - 1 : off[a];
                    Vector fc(grid.CoordinateX[idx[0]], grid.CoordinateY[idx[1]], grid.CoordinateZ[idx[2]]);
                    const double* H = a == 0 ? &grid.hx[0] : (a == 1 ? &grid.hy[0] : &grid.hz[0]);
                    const double hh = 0.5 * H[idx[a]] * (hi ? 1.0 : -1.0);
                    if (a == 0) fc.x += hh;
                    else if (a == 1) fc.y += hh;
                    else fc.z += hh;
                    const int mk = sides[s]->getMarker(fc);
                    auto it = kind_of_marker.find(mk);
                    if (it == kind_of_marker.end()) {
                        if ((int)kind_of_marker.size() == TS_MAX_BC_KINDS)
                            throw std::runtime_error("more distinct boundary markers than TS_MAX_BC_KINDS");
                        const int k = (int)kind_of_marker.size();
                        cfg.bc_kinds[k] = to_bc(c.MyConditions.at(mk));
                        it = kind_of_marker.emplace(mk, k).first;
                    }
                    marks[s].push_back((uint8_t)it->second);
                }
            cfg.bc_marker[s] = marks[s].data();
        }
        cfg.n_bc_kinds = (int32_t)kind_of_marker.size();
        return cfg;
    }

    void InitializeMethod(KernelConfiguration& c) override {
        cfg_ = MakeConfig(c, grid, precision_, device_, blocks_, marks_);
        if (h_) ts_destroy(h_);
        h_ = nullptr;
        check(ts_create(&cfg_, &h_));
        stepInfo.Residual.resize(nVariables, 0.0);
        host_newer_ = true;
        device_newer_ = false;
    }

    void IterationStep() override {
        if (host_newer_) SyncToDevice();
        // snapshot times Run advanced on the host (kernel.h:1777, :1796)
        ts_step_info si{};
        check(ts_get_step_info(h_, &si));
        if (si.next_solution_time != stepInfo.NextSolutionSnapshotTime ||
            si.next_slice_time != stepInfo.NextSliceSnapshotTime || si.time != stepInfo.Time ||
            si.iteration != stepInfo.Iteration) {
            si.time = stepInfo.Time;
            si.iteration = stepInfo.Iteration;
            si.next_solution_time = stepInfo.NextSolutionSnapshotTime;
            si.next_slice_time = stepInfo.NextSliceSnapshotTime;
            check(ts_set_step_info(h_, &si));
        }
        check(ts_step(h_, 1, &si));
        device_newer_ = true;
        stepInfo.Time = si.time;
        stepInfo.TimeStep = si.dt;
        stepInfo.Iteration = si.iteration;
        stepInfo.Residual.resize(nVariables, 0.0);
        for (int v = 0; v < nVariables && v < 5; ++v) stepInfo.Residual[v] = si.residual[v];
        if (si.health) throw std::runtime_error("non-physical state on the GPU (health flags " +
                                                std::to_string(si.health) + ")");
        if (reader_due()) SyncFromDevice();
    }

    void SaveSolutionToTecplot(std::string fname) override {
        SyncFromDevice();
        Kernel::SaveSolutionToTecplot(fname);
    }

    // Host `values` -> device (after the host wrote them).
    void SyncToDevice() {
        check(ts_set_state(h_, &values[0], TS_LAYOUT_WITH_GHOSTS));
        host_newer_ = false;
        device_newer_ = false;
    }
    // Device -> host `values`, if the device is ahead.
    void SyncFromDevice() {
        if (!device_newer_) return;
        check(ts_get_state(h_, &values[0], TS_LAYOUT_WITH_GHOSTS));
        device_newer_ = false;
    }
    ts_handle* Handle() const { return h_; }
    const ts_config& Config() const { return cfg_; }

private:
    static ts_bc_config to_bc(const BoundaryConditionConfiguration& b) {
        ts_bc_config r{};
        r.type = (int32_t)b.BCType;
        r.density = b.Density;
        r.velocity[0] = b.Velocity.x;
        r.velocity[1] = b.Velocity.y;
        r.velocity[2] = b.Velocity.z;
        r.pstatic = b.Pstatic;
        r.temperature = b.Temperature;
        return r;
    }
    static void check(ts_status s) {
        if (s != TS_OK) throw std::runtime_error(std::string("libtsfvm: ") + ts_last_error());
    }
    // The Run loop reads `values` after this step (kernel.h:1720-1846).
    bool reader_due() const {
        const int it = stepInfo.Iteration;
        if (isSensorEnable && SaveSensorRecordIters > 0 && it % SaveSensorRecordIters == 0) return true;
        if (SaveSolutionIters != 0 && it % SaveSolutionIters == 0) return true;
        if (SaveSliceIters != 0 && it % SaveSliceIters == 0) return true;
        if (SaveBinarySolIters != 0 && it % SaveBinarySolIters == 0) return true;
        if (SaveSolutionTime > 0 && stepInfo.NextSolutionSnapshotTime == stepInfo.Time) return true;
        if (SaveSliceTime > 0 && stepInfo.NextSliceSnapshotTime == stepInfo.Time) return true;
        return it == MaxIteration || stepInfo.Time >= MaxTime;
    }

    int precision_, device_;
    ts_handle* h_ = nullptr;
    ts_config cfg_{};
    std::vector<ts_block_node> blocks_[3];
    std::vector<uint8_t> marks_[6];
    bool host_newer_ = true;
    bool device_newer_ = false;
};

// CreateKernel (ExplicitRungeKuttaFVM.h:1496-1513) for the GPU: null for a
// configuration libtsfvm.so does not build (the reference returns null for
// reconstructions it has no kernel for).
inline std::unique_ptr<Kernel> CreateGpuKernel(KernelConfiguration& conf, int argc, char* argv[],
                                               int precision = TS_PRECISION_MIXED, int device = 0) {
    if (conf.SolutionMethod != KernelConfiguration::Method::ExplicitRungeKuttaFVM) return nullptr;
    if (conf.DummyLayerSize != 1) return nullptr;  // the reference's stencil assumes one ghost layer
    return std::unique_ptr<Kernel>(new GpuExplicitRungeKuttaFVM(&argc, &argv, precision, device));
}

#endif
