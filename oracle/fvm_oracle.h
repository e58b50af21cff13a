/*
 * TEST INFRASTRUCTURE ONLY.  CPU restatement of the reference solver's explicit
 * finite-volume step (TurboStructred, src/Methods/ExplicitRungeKuttaFVM.h and
 * the plugins it calls), used as the parity checker for the CUDA path and as
 * the timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU legs may load it; the product library never links or calls it.
 *
 * Parity is pinned: tests/test_oracle_pinned.py checks this restatement
 * bit-for-bit against the reference's own code (compiled from its sources into
 * oracle/_ref/ by oracle/ref_build/Makefile) through the committed fixtures in
 * tests/golden/.  HLLC and the stiffened-gas EOS are not in the reference: for
 * those the oracle is this restatement alone ("parity unpinned by the
 * reference"), checked against exact Riemann solutions instead.
 *
 * State layout is the reference's own `values` array (kernel.h:88-96,
 * grid.h:64-67): one ghost layer on every active axis, cells x-fastest, the 5
 * conserved variables (rho, rho*u, rho*v, rho*w, rho*E) contiguous per cell.
 */
#ifndef TS_FVM_ORACLE_H
#define TS_FVM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_BLOCKS 16
#define ORC_MAX_BC_KINDS 8
#define ORC_BC_IDS (6 + ORC_MAX_BC_KINDS)

enum { ORC_RECON_PWC = 0, ORC_RECON_LINEAR2 = 1, ORC_RECON_ENO2 = 2, ORC_RECON_LINEAR2_LIM = 3 };
enum { ORC_LIM_BJ = 0, ORC_LIM_VENKAT = 1 };
enum { ORC_RS_GODUNOV = 0, ORC_RS_ROE = 1, ORC_RS_NONE = 2, ORC_RS_HLLC = 3 };
enum { ORC_BC_WALL = 0, ORC_BC_SYMMETRY = 1, ORC_BC_MOVING_WALL = 2, ORC_BC_SUBSONIC_INLET = 3,
       ORC_BC_SUBSONIC_OUTLET = 4, ORC_BC_NATURAL = 5 };
enum { ORC_EOS_IDEAL = 0, ORC_EOS_STIFFENED = 1 };

typedef struct {
    int ndims, nx, ny, nz;
    int periodic[3];
    double length[3];
    /* Optional stretched blocks per axis (KernelConfiguration.h:10-19,37-39);
       n_blocks[a] == 0 means one uniform block. */
    int n_blocks[3];
    double block_pos[3][ORC_MAX_BLOCKS];
    double block_q[3][ORC_MAX_BLOCKS];
    int block_cells[3][ORC_MAX_BLOCKS];
    double gamma;
    int eos;
    double p_inf;
    int recon, limiter, solver;
    double eps, cfl;
    int max_iteration;
    double max_time, save_solution_time, save_slice_time;
    /* BC table: entries 0-5 per side xL,xR,yL,yR,zL,zR, entries 6.. the
       extra kinds (KernelConfiguration::MyConditions entries): a
       BoundaryConditionType and its parameters
       (BoundaryConditionConfiguration.h:21-35). */
    int bc_type[ORC_BC_IDS];
    double bc_density[ORC_BC_IDS], bc_velocity[ORC_BC_IDS][3], bc_pstatic[ORC_BC_IDS];
    int threads; /* OpenMP threads (0 = runtime default) */
    /* Source terms: IsExternalForceRequared with Sigma, IsUnifromAccelerationRequared
       with UniformAcceleration (KernelConfiguration.h:50-51,87-88). */
    int external_force, uniform_acceleration;
    double sigma[3], acceleration[3];
    /* Viscous flow: IsViscousFlow and Viscosity (KernelConfiguration.h:43,49).
       The viscosity enters the spectral radius even when viscous == 0
       (ExplicitRungeKuttaFVM.h:1239-1248). */
    int viscous;
    double viscosity;
    /* Position-dependent sides (DomainBCinfo::isComplex / getMarker,
       BoundaryConditionConfiguration.h:43-66): per boundary face the extra
       kind (entry 6 + marker) it takes, faces numbered by the tangential
       interior cell indices, lower axis fastest; NULL: the side's own BC. */
    const unsigned char* bc_marker[6];
} orc_config;

typedef struct {
    int iteration;
    double time, dt;
    double next_solution_time, next_slice_time;
    double residual[5];
} orc_step_info;

/* Cell counts of the reference's values array including ghosts. */
void orc_dims(const orc_config* c, int* nx_all, int* ny_all, int* nz_all);

/* Cell centres and sizes per axis including ghosts (grid.h:124-344). */
int orc_grid(const orc_config* c, double* x, double* hx, double* y, double* hy, double* z, double* hz);

/* Advance `values` (full array with ghosts) by n_steps IterationStep calls,
   or, when n_steps < 0, by the Kernel::Run loop until MaxIteration or
   MaxTime (kernel.h:1701-1850).  `info` carries time/iteration in and out.
   Returns 0 on success. */
int orc_advance(const orc_config* c, double* values, int n_steps, orc_step_info* info);

/* Exact Riemann solution sampled at x/t = s for a stiffened (p_inf >= 0)
   gas; Toro, "Riemann Solvers and Numerical Methods for Fluid Dynamics",
   ch. 4 pressure-function method with the stiffened-gas substitution
   p -> p + p_inf.  Outputs primitive rho,u,p.  Returns iterations used. */
int orc_exact_riemann(double gamma, double p_inf, double rl, double ul, double pl, double rr,
                      double ur, double pr, double s, double* rho, double* u, double* p);

/* Star pressure of the ideal-gas Riemann problem by Newton-Raphson (the
   Godunov flux's inner solve); returns 1 when converged. */
int orc_godunov_pstar(double gamma, double rl, double ul, double pl, double rr, double ur, double pr, double* ps);

/* The benchmark scenarios' initial states (interior cells, x fastest, 5
   doubles per cell) and their hash RNG: uniform double in [0,1) of
   (seed, i, j, k).  Scenario 0 shock tube, 1 shear layer, 2 blast,
   3 quadrants; parameters as ts_fill_scenario.  Returns 0 on success. */
double orc_hash_uniform(unsigned long long seed, long long i, long long j, long long k);
int orc_fill_scenario(const orc_config* c, int scenario, unsigned long long seed, const double* params, int n_params,
                      double* values);

#ifdef __cplusplus
}
#endif
#endif
