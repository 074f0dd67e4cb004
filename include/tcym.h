/*
 * tcym.h — C ABI of the GB300-native real-time lattice Yang-Mills hot path
 * (SU(2)/SU(3) on a periodic 3D lattice): the drop-in for the GaugeLinks /
 * ElectricFields objects and the Dynamics, LangevinDynamics, GradientFlow,
 * GaussLawRestoration, Observables and Chern-Simons-rate calls of
 * markmace/TopologicalCYMSolver.
 *
 * Plain C: opaque handles, pointers and sizes, int status codes.  Host arrays
 * passed to upload/download use the reference's own AoS FP64 layouts:
 *   U: V*3*NMD doubles, link (x,y,z,mu) at NMD*(mu + 3*site), NMD = 4 for SU(2)
 *      (u0,u1,u2,u3 with U = u3 + i u_k sigma_k) or 18 for SU(3) (9 complex,
 *      column-major (i,j) -> i + 3j)          (LATTICE/GaugeLinks.cpp:27-47)
 *   E: V*3*NA doubles, E^a_mu(x) at a + NA*(mu + 3*site), NA = 3 or 8
 *                                             (LATTICE/ElectricFields.cpp:36-46)
 *   site = x + Nx*(y + Ny*z)
 * The device copy is private to the library (structure-of-arrays; FP32 or FP64).
 *
 * Threading: a context owns a CUDA device; every lattice has its own stream.
 * Calls on different lattices may run concurrently from different threads;
 * calls on one lattice must be serialised by the caller.  No call exits or
 * aborts: every failure is a status code with a message in tcym_last_error().
 */
#ifndef TCYM_H
#define TCYM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TCYM_VERSION 100

/* status codes */
enum {
    TCYM_OK = 0,
    TCYM_ERR_ARG = 1,        /* invalid argument */
    TCYM_ERR_OOM = 2,        /* device allocation failed */
    TCYM_ERR_CUDA = 3,       /* CUDA runtime error (message has the CUDA string) */
    TCYM_ERR_NONFINITE = 4,  /* a reduction saw NaN/Inf: the state is unhealthy */
    TCYM_ERR_TIMEOUT = 5,    /* a bounded wait on device progress ran out */
    TCYM_ERR_ADMISSION = 6,  /* the serving loop refused a request (HBM budget) */
    TCYM_ERR_STATE = 7       /* call not valid in the object's state */
};

/* storage precision of a lattice */
enum {
    TCYM_FP64 = 0, /* FP64 links and fields: the plain drop-in */
    TCYM_FP32 = 1  /* FP32 storage (SU(3): two rows), FP64 reductions and reunitarisation */
};

/* E.B operator of the Chern-Simons rate in calibrated flow */
enum {
    TCYM_NCS_IMPROVED = 1, /* O(a^2)-improved, the reference's NCsDot default */
    TCYM_NCS_CLOVER = 2    /* clover (UnimprovedOperators) */
};

/* gradient-flow sweep order */
enum {
    TCYM_FLOW_SIMULTANEOUS = 0, /* all links at once, as GradientFlow::StandardUpdate */
    TCYM_FLOW_CHECKERBOARD = 1  /* six in-place sub-sweeps by (site parity, direction) */
};

typedef struct tcym_ctx_s *tcym_ctx;
typedef struct tcym_lattice_s *tcym_lattice;

/* FP64 observables of one lattice (all spacings 1 -> metric factors 1):
 * Observables::Bulk (OBSERVABLES/BulkObservables.cpp:29-143),
 * Observables::GaussLaw (GaussLawViolation.cpp:13-61),
 * Observables::Unitarity (UnitarityViolation.cpp:13-51),
 * UnimprovedOperators::ComputeEDotB (CALC/ChernSimonsOperators.cpp:4-47). */
typedef struct {
    double T00;          /* energy density: Bulk::T00() */
    double electric;     /* Bulk::ELECTRIC() */
    double magnetic;     /* Bulk::MAGNETIC() */
    double esqr[3];      /* Bulk::ESqr[mu]: <sum_a E^a_mu E^a_mu> */
    double bsqr[3];      /* Bulk::BSqr[i]:  <4 Re tr(1 - P_jk)> */
    double gauss_max;    /* GaussLaw::GlobalMaxViolation (signed maximum, from 0) */
    double gauss_rms;    /* GaussLaw::GlobalAvgViolation */
    double gauss_absmax; /* max |G^a(x)| (no reference counterpart) */
    double unit_max;     /* Unitarity::GlobalMaxViolation */
    double unit_rms;     /* Unitarity::GlobalAvgViolation */
    double edotb;        /* sum_x E.B with the clover operator */
    double ncs_dot;      /* edotb / (8 pi^2): ChernSimonsNumber::NCsDot (TOPOLOGY/ChernSimonsDerivative.cpp:31-49) */
    double ncs;          /* Kahan-compensated integral of ncs_dot dt tracked during steps */
    int nonfinite;       /* 1 when any reduced quantity was NaN/Inf */
} tcym_obs;

int tcym_version(void);

/* ---------------------------------------------------------------- context */
/* Opens a context on CUDA device `device`. */
int tcym_ctx_create(int device, tcym_ctx *out);
int tcym_ctx_destroy(tcym_ctx ctx);
/* Message of the last failure on this context (valid until the next call). */
const char *tcym_last_error(tcym_ctx ctx);

/* ---------------------------------------------------------------- lattices */
/* GaugeLinks(Nx,Ny,Nz,ax,ay,az) + ElectricFields(...) (LATTICE/GaugeLinks.cpp:65-81,
 * LATTICE/ElectricFields.cpp:66-82): allocates links (ping-pong pair) and fields on the
 * device.  nc = 2 or 3; spacings a = 1. Contents are undefined until set. */
int tcym_lattice_create(tcym_ctx ctx, int nc, int nx, int ny, int nz, int precision, tcym_lattice *out);
/* as tcym_lattice_create with lattice spacings a[3] (reference: integer spacings). */
int tcym_lattice_create_ex(tcym_ctx ctx, int nc, int nx, int ny, int nz, const double a[3], int precision,
                           tcym_lattice *out);
int tcym_lattice_destroy(tcym_lattice lat);
/* device bytes held by the lattice (links, fields, scratch) */
int tcym_lattice_bytes(tcym_lattice lat, size_t *bytes);
/* Copies host AoS FP64 arrays in (either may be NULL), converting to the storage format. */
int tcym_lattice_upload(tcym_lattice lat, const double *U_aos, const double *E_aos);
/* Copies the state out to host AoS FP64 arrays (either may be NULL). */
int tcym_lattice_download(tcym_lattice lat, double *U_aos, double *E_aos);
/* One leapfrog step (Dynamics::Update, DYNAMICS/Dynamics.cpp:204-218) of a state held in host memory:
 * U_in/E_in in, U_out/E_out out, in the AoS layouts of tcym_lattice_upload (U_out may be U_in, E_out
 * E_in).  The upload, the step and the download run as one pipeline over z-ordered chunks, so both
 * transfer directions overlap each other and the step; the lattice holds the new state afterwards,
 * as after tcym_lattice_upload + tcym_leapfrog(lat, dt, 1) + tcym_lattice_download, bit for bit.
 * Host buffers in pinned memory (cudaMallocHost / cudaHostRegister) make the copies asynchronous. */
int tcym_leapfrog_host(tcym_lattice lat, double dt, const double *U_in, const double *E_in, double *U_out,
                       double *E_out);
/* Block(GaugeLinks**) + Block(ElectricFields**) (LATTICE/GaugeLinks.cpp:124-145,
 * LATTICE/ElectricFields.cpp:113-127) into dst, a lattice of the same group and
 * precision with half the (even) extents of src: dst's links become
 * U'_mu(x) = U_mu(2x) U_mu(2x + mu) (products in FP64), its fields zero and its
 * spacings twice src's. */
int tcym_lattice_block(const tcym_lattice src, tcym_lattice dst);
/* dst <- src: links, fields and spacings (same group and extents; any precisions): Copy() of GaugeLinks.cpp:91-107
 * and ElectricFields.cpp:90-104. */
int tcym_lattice_copy(tcym_lattice dst, const tcym_lattice src);
/* Binary snapshot of the lattice for an exact resume (no reference counterpart in binary form:
 * the reference checkpoints only through its 15-digit configuration text files,
 * IO/SaveConfiguration.cpp:3-56, which tcym_lattice_save writes).  The snapshot holds the links
 * and fields in the device's own storage format, bit for bit, plus the step count, the
 * reunitarisation phase, the N_CS tracking period, the Kahan-compensated N_CS pair, the
 * ping-pong parity and the Langevin noise stream (seed and next step of the last tcym_langevin
 * call).  Restoring into a lattice of the same group, precision and extents (spacings are taken
 * from the snapshot) and stepping on gives the same bits as never having stopped.
 * tcym_lattice_snapshot_bytes: size of the snapshot; tcym_lattice_snapshot: into a host buffer
 * of at least that size; tcym_lattice_restore: from one (TCYM_ERR_ARG for another lattice's
 * snapshot, a truncated one or a checksum mismatch).  The _file forms go through a file. */
int tcym_lattice_snapshot_bytes(tcym_lattice lat, size_t *bytes);
int tcym_lattice_snapshot(tcym_lattice lat, void *buf, size_t bytes);
int tcym_lattice_restore(tcym_lattice lat, const void *buf, size_t bytes);
int tcym_lattice_snapshot_file(tcym_lattice lat, const char *path);
int tcym_lattice_restore_file(tcym_lattice lat, const char *path);
/* The Langevin noise stream of the lattice's last tcym_langevin call: its seed and the first step
 * not yet drawn (valid = 0 before any Langevin step); restored with a snapshot. */
int tcym_lattice_noise_state(tcym_lattice lat, uint64_t *seed, uint64_t *next_step, int *valid);
/* Steps taken by the lattice (leapfrog, Langevin, simultaneous flow) since it was created. */
int tcym_lattice_steps(tcym_lattice lat, int64_t *steps);
/* Waits for all work queued on the lattice. */
int tcym_lattice_sync(tcym_lattice lat);
/* The lattice's CUDA stream (a cudaStream_t), for ordering or timing caller work
 * against the library's kernels. */
int tcym_lattice_stream(tcym_lattice lat, void **stream);
/* Page-locked host memory (cudaMallocHost) for the host arrays of tcym_lattice_upload / _download and
 * tcym_leapfrog_host, whose copies then run asynchronously (and, for the host-resident step, overlap
 * each other); for callers that do not link the CUDA runtime themselves.  Freed with tcym_host_free. */
int tcym_host_alloc(size_t bytes, void **ptr);
int tcym_host_free(void *ptr);

/* ------------------------------------------------------ initial conditions */
/* InitialConditions::SetZero (INITIALCONDITIONS/SetZero.cpp:3-24): U = 1, E = 0. */
int tcym_set_zero(tcym_lattice lat);
/* E^a_mu(x) = sigma * N(0,1) from the Philox field stream of `seed`; with
 * sigma = 1/sqrt(beta) this is ThermalDynamics::ReassignElectricFields before its
 * Gauss restore (DYNAMICS/ThermalDynamics.cpp:205-226). */
int tcym_gaussian_efield(tcym_lattice lat, double sigma, uint64_t seed);
/* ThermalDynamics::Thermalize(rounds, max_time) (DYNAMICS/ThermalDynamics.cpp:260-314):
 * `rounds` times, E = N(0,1)/sqrt(beta) (round r: field stream step r), Gauss
 * restore (restore_tol <= 0: 1e-14 in FP64, 1e-6 in FP32; at most 10000 sweeps),
 * then leapfrog steps of dt while steps*dt < max_time (the reference: dt 0.0375).
 * Every `every` steps (the reference: 20) one record of 7 doubles is written to
 * series (up to series_cap records; *records gets the count): t + r*max_time,
 * T00, TXX, TYY, TZZ, ELECTRIC, MAGNETIC, the reference's ThermalEnergy line. */
int tcym_thermalize(tcym_lattice lat, double beta, uint64_t seed, int rounds, double max_time, double dt,
                    double restore_tol, int every, double *series, int series_cap, int *records);

/* Block tiling of the packed FP32 step (FP32 lattices with even nz; no reference
 * counterpart): each block of 128 threads advances tx x ty site pairs of one z-plane,
 * or, for tx = 0, 128 consecutive pairs.  Chosen on the lattice's first step by an
 * autotuner that times the candidates on a proxy lattice with the same nx, ny (at most
 * 1 GiB), cached per format and extents in the context; TCYM_TILE=linear
 * or TCYM_TILE=<tx>x<ty> in the environment overrides it.  Results do not depend on
 * the tiling.  tcym_lattice_set_tile fixes it (tx a power of two, tx * ty = 128, or
 * tx = 0) or, with tx = -1, hands it back to the autotuner. */
int tcym_lattice_tile(tcym_lattice lat, int *tx, int *ty);
int tcym_lattice_set_tile(tcym_lattice lat, int tx, int ty);

/* ---------------------------------------------------- cooled Chern-Simons number
 * ChernSimonsNumber::CoolingMethod (TOPOLOGY/CoolingMethod.cpp).  The object holds
 * the last two cooled copies UOld, UNew of the lattice's links; a copy is made as
 * Cooling::CoolNSave does (GRADIENTFLOW/Cooling.cpp:69-175): max_steps
 * GradientFlow::StandardUpdate steps of DcTau = sqrt_dctau^2 (a_x a_y a_z)^(2/3) from
 * E = 0 (the reference: 128 steps, SphaleronSimulation.cpp:230).  With a blocking
 * level L > 0 (StandardBlockingLevel) links and fields are blocked (tcym_lattice_block)
 * after steps block_frequency * 8^b, b < L (Cooling::BlockFrequency), so the cooled
 * copies have the extents divided by 2^L: the extents must be divisible by 2^L and
 * block_frequency * 8^(L-1) <= max_steps.  tcym_cooling_create is level 0, the level of
 * the reference's real-time measurement (SphaleronSimulation.cpp:230-236).  The lattice
 * is only read. */
typedef struct tcym_cooling_s *tcym_cooling;
int tcym_cooling_create(tcym_lattice lat, int max_steps, double sqrt_dctau, tcym_cooling *out);
int tcym_cooling_create_ex(tcym_lattice lat, int max_steps, double sqrt_dctau, int blocking_level,
                           int block_frequency, tcym_cooling *out);
int tcym_cooling_destroy(tcym_cooling c);
/* CoolingMethod::Start (:124-135): UNew = the cooled links, UOld = UNew. */
int tcym_cooling_start(tcym_cooling c);
/* CoolingMethod::Update(measure) (:141-166): UNew = the cooled links; if measure,
 * delta = GetDeltaNCs(1) on the geodesic UOld -> UNew is added to the running total
 * (DeltaNCsCoolRealTime) and returned in *delta (nullable); then UOld = UNew.
 * TCYM_ERR_STATE before tcym_cooling_start. */
int tcym_cooling_update(tcym_cooling c, int measure, double *delta);
/* CoolingMethod::GetDeltaNCs(norder) (:77-120) on the current UOld, UNew: Simpson's
 * rule along the geodesic EMid = -i Log(UNew UOld^dag), UMid(x) = exp(-i x EMid) UOld
 * (SUNc/AdvancedOperations.cpp:432-442) of NCsDot = improved E.B / (8 pi^2). */
int tcym_cooling_delta_ncs(tcym_cooling c, int norder, double *out);
/* the sum of the measured updates (ChernSimonsNumber::DeltaNCsCoolRealTime) */
int tcym_cooling_total(tcym_cooling c, double *out);
/* the latest cooled links (CoolingMethod::UOld, blocked to the extents divided by
 * 2^level) in the reference's AoS layout; TCYM_ERR_STATE before tcym_cooling_start. */
int tcym_cooling_links(tcym_cooling c, double *U_aos);

/* ------------------------------------------------------- configuration files
 * The reference's text format (IO/SaveConfiguration.cpp:3-56, IO/LoadConfiguration.cpp:3-120):
 * a link file with one line "x y z mu v_0 .. v_{n-1} " per link (SU(2): 4 reals; SU(3):
 * re, im of the 9 entries in storage order) and a field file with one line
 * "x y z mu e^0 .. e^{NA-1}" per link, z-, y-, x-, mu-major, 15 significant digits.
 * Host arrays in the reference AoS layouts (as tcym_lattice_upload).  Either file may be
 * NULL.  Reading accepts lines in any order but needs every link exactly once
 * (TCYM_ERR_ARG otherwise, with the reason on stderr; the reference exits instead). */
int tcym_write_configuration(int nc, int nx, int ny, int nz, const double *U_aos, const double *E_aos,
                             const char *ufile, const char *efile);
int tcym_read_configuration(int nc, int nx, int ny, int nz, double *U_aos, double *E_aos, const char *ufile,
                            const char *efile);
/* the lattice's state to / from such files (through tcym_lattice_download / _upload) */
int tcym_lattice_save(tcym_lattice lat, const char *ufile, const char *efile);
int tcym_lattice_load(tcym_lattice lat, const char *ufile, const char *efile);
/* U_mu(x) = exp(i t^a theta^a), theta^a = sigma * N(0,1) from the Philox link stream. */
int tcym_random_links(tcym_lattice lat, double sigma, uint64_t seed);
/* GaussLawRestoration::Restore (GAUSSLAWFIXING/GaussRestore.cpp:131-167): iterate
 * E -= g (G(x) - Adj(U) G(x+mu)), g = 7/24, 7/48, 7/72, until the signed maximum
 * of G is <= tol (reference: 1e-14) or maxit iterations (reference: 10000).
 * iters / final_max may be NULL. */
int tcym_gauss_restore(tcym_lattice lat, double tol, int maxit, int *iters, double *final_max);
/* Same restore, run in place on caller-owned device buffers in the AoS FP64 layouts
 * above, without allocating any memory.  It has no counterpart in the reference.
 * It is for callers that cannot let a library call cudaMalloc: their device memory is
 * wholly reserved by their own allocator, or they run a steady-state loop in which
 * cudaFree's device-wide synchronisation or a cudaMalloc failure cannot happen.
 * U_aos (read) and E_aos (updated) are device pointers on the current device; `stream`
 * is a cudaStream_t (NULL = the default stream); iters / final_max as above (may be
 * NULL); errbuf receives a message on failure (may be NULL).
 * Scratch is a fixed 8 MiB device array inside libtcym.so.  It is reserved on a device
 * when the library's module that holds it loads there, which with lazy module loading
 * is the first call of this entry point on that device; that first call also loads the
 * code of the kernels it runs, for both groups.  Make the first call on each device
 * before the caller's allocator reserves that device's memory, or it can fail for lack
 * of memory.  Later calls allocate nothing; the reservation lasts until the process exits.
 * Lattices whose violation array (NA * V doubles) exceeds 1,036,272 doubles are rejected
 * with TCYM_ERR_ARG: SU(2) at most 345,424 sites, SU(3) at most 129,534 sites.
 * Every call reads results back to the host and synchronises `stream` once per
 * iteration, so no call may run while its stream is being captured into a graph.
 * All calls share the one scratch array, which keeps the last call's contents (each
 * call clears what must start at zero): calls that overlap on the GPU, from any thread
 * or stream, race and must not be issued.
 * TCYM_ERR_NONFINITE: a reduction saw NaN or Inf in U or E (E is left as it was at that
 * iteration). */
int tcym_gauss_restore_noalloc(int nc, int nx, int ny, int nz, const double *U_aos, double *E_aos, double tol,
                               int maxit, void *stream, int *iters, double *final_max, char *errbuf, size_t errlen);

/* --------------------------------------------------------------- dynamics */
/* Dynamics::Update(U,E) (DYNAMICS/Dynamics.cpp:204-218), nsteps times: E update from
 * the plaquettes (Dynamics.cpp:145-197) then U <- exp(-i dt E) U (Dynamics.cpp:97-138),
 * fused in one kernel per step. */
int tcym_leapfrog(tcym_lattice lat, double dt, int nsteps);
/* Dynamics::UpdateElectricFields over the whole lattice (Dynamics.cpp:145-197). */
int tcym_update_e(tcym_lattice lat, double dt);
/* Dynamics::UpdateGaugeLinks over the whole lattice (Dynamics.cpp:97-138). */
int tcym_update_u(tcym_lattice lat, double dt);
/* LangevinDynamics::Update() without its periodic prints (DYNAMICS/LangevinDynamics.cpp:
 * 260-347): E += dt F - gamma dt E + sqrt(gamma dt) sqrt(2T) xi, then the link update,
 * for steps step0 .. step0+nsteps-1.  xi ~ N(0,1) drawn in-kernel from the Philox noise
 * stream keyed by (seed, step, site, mu, colour).  The reference has gamma = 1 and
 * beta = 1/T (LangevinDynamics.cpp:23,184-186). */
int tcym_langevin(tcym_lattice lat, double dt, double gamma, double T, uint64_t seed, uint64_t step0, int nsteps);
/* GradientFlow::StandardUpdate (calibrate = 0) / CalibrationUpdate (calibrate =
 * TCYM_NCS_IMPROVED or TCYM_NCS_CLOVER) (GRADIENTFLOW/GradientFlow.cpp:150-188), nsteps
 * flow steps of size dtau (the reference's DcTau = SqrtDcTauOverSpacing^2 (a_x a_y a_z)^(2/3),
 * GradientFlow.cpp:150; calibration: unit spacings), all links at
 * once or checkerboarded.  With calibrate, *dncs receives sum dtau/2 [NCsDot(U,F) +
 * NCsDot(U',F)] with the chosen E.B operator (the reference uses the improved one).
 * In checkerboard mode F is the force of the state before each sweep.  The field array
 * holds the last flow force afterwards, as in the reference.  Checkerboard mode needs
 * even extents. */
int tcym_flow(tcym_lattice lat, double dtau, int nsteps, int mode, int calibrate, double *dncs);
/* Projects every stored link back onto the group in FP64 (no reference counterpart). */
int tcym_reunitarize(tcym_lattice lat);
/* Reunitarise automatically every `period` steps of leapfrog/Langevin (0 = never).
 * Default: 100 for TCYM_FP32 lattices, 0 for TCYM_FP64. */
int tcym_set_reunitarize_period(tcym_lattice lat, int period);

/* ------------------------------------------------------------ observables */
/* All observables of the current state (FP64 reductions, fixed order). Returns
 * TCYM_ERR_NONFINITE (with *out filled) when a reduced value is NaN/Inf. */
int tcym_observables(tcym_lattice lat, tcym_obs *out);
/* UnimprovedOperators::ComputeEDotB (CALC/ChernSimonsOperators.cpp:4-47): sum_x E.B, clover. */
int tcym_edotb(tcym_lattice lat, double *out);
/* ImprovedOperators::ComputeEDotB (CALC/ChernSimonsOperators.cpp:72-382): sum_x E.B with
 * the O(a^2)-improved fields (4 boxes + 8 rectangles, 4-point transported E). */
int tcym_edotb_improved(tcym_lattice lat, double *out);
/* Track N_CS during leapfrog/Langevin steps: every `every` steps (0 = off) add
 * every*dt * NCsDot of the new state to a Kahan-compensated FP64 sum on the device. */
int tcym_ncs_track(tcym_lattice lat, int every);
int tcym_ncs_get(tcym_lattice lat, double *ncs);
int tcym_ncs_reset(tcym_lattice lat);

/* --------------------------------------------------------------- ensembles */
/* Many independent lattices advanced together: the trajectories the reference
 * runs as independent MPI ranks sharing only a seed (SU2Solver.cpp:161-164,
 * SphaleronSimulation.cpp:571-616).  Members may mix groups, sizes, precisions
 * and dynamics.  Each step is one persistent batched launch per storage format
 * present; tcym_ensemble_step captures its chunk of steps as a CUDA graph and
 * replays it while membership and chunk length are unchanged.  A member's
 * arithmetic is the same as when it is stepped alone.  While a lattice is a
 * member, step it only through the ensemble; other calls on it are fine
 * between ensemble calls (tcym_ensemble_step returns after the work is done). */
typedef struct tcym_ensemble_s *tcym_ensemble;
enum { TCYM_DYN_LEAPFROG = 0, TCYM_DYN_LANGEVIN = 1 };
int tcym_ensemble_create(tcym_ctx ctx, tcym_ensemble *out);
int tcym_ensemble_destroy(tcym_ensemble ens);
/* Adds a member with its own dynamics: leapfrog (dt) or Langevin (dt, gamma, T,
 * noise seed, first noise step).  Members keep the order they were added in. */
int tcym_ensemble_add(tcym_ensemble ens, tcym_lattice lat, int dynamics, double dt, double gamma, double T,
                      uint64_t seed, uint64_t step0);
int tcym_ensemble_remove(tcym_ensemble ens, tcym_lattice lat);
/* How the ensemble's FP32 site-pair members step (no reference counterpart; the reference runs
 * each trajectory as its own process).  group_blocks < 0 (the default): one batched launch per
 * step (graph-captured chunks).  group_blocks >= 0: one persistent launch per chunk of K steps and
 * coefficient class, whose blocks take (member block, step) work items in order and wait, with a
 * time limit, only for the member's own previous step; members are cut into groups of at least
 * group_blocks blocks (0: one group) and a group runs all K steps before the next.
 * Results are the same bits either way.  Applies from the next tcym_ensemble_step. */
int tcym_ensemble_set_persistent(tcym_ensemble ens, int group_blocks);
int tcym_ensemble_size(tcym_ensemble ens, int *n);
/* Advances every member nsteps steps. */
int tcym_ensemble_step(tcym_ensemble ens, int nsteps);
/* Clover E.B of every member (sum_x E.B, member order) in one batched reduction.
 * With ncs_stride > 0 each member's Kahan N_CS advances by ncs_stride*dt*E.B/(8 pi^2)
 * (a measurement every ncs_stride steps); ncs receives the running N_CS.  Either
 * output may be NULL. */
int tcym_ensemble_measure(tcym_ensemble ens, int ncs_stride, double *edotb, double *ncs);

/* ------------------------------------------------------------------ serving */
/* A request loop with continuous batching (the reference's one-trajectory-per-
 * process drivers, SphaleronSimulation.cpp:571-616, LangevinSimulationSU3.cpp:469-512,
 * as a service).  A background thread admits requests in arrival order while the
 * device-memory budget and the slot limit allow, advances all admitted requests
 * together (an ensemble, `stride` steps per tick), records each request's N_CS
 * every `stride` steps, and retires finished requests at once, freeing their
 * memory for the next arrivals.  Initial state of a request: U = 1, E ~ N(0, T)
 * per component from the Philox field stream of its seed, Gauss-restored.
 * N_CS is the Kahan sum of stride*dt*NCsDot (clover) sampled at the end of each
 * tick.  Results do not depend on which other requests share the device. */
typedef struct tcym_server_s *tcym_server;
typedef struct {
    int nc;         /* 2 or 3 */
    int L;          /* cubic extent */
    int precision;  /* TCYM_FP32 or TCYM_FP64 */
    int dynamics;   /* TCYM_DYN_LEAPFROG or TCYM_DYN_LANGEVIN */
    double dt;      /* time step */
    double gamma;   /* Langevin damping (ignored for leapfrog) */
    double T;       /* initial E variance and Langevin temperature */
    int nsteps;     /* steps; rounded up to a multiple of the server's stride */
    uint64_t seed;  /* Philox seed of the initial fields and of the noise */
} tcym_request;
enum { TCYM_REQ_QUEUED = 0, TCYM_REQ_RUNNING = 1, TCYM_REQ_DONE = 2, TCYM_REQ_FAILED = 3 };
typedef struct {
    int queued, active;
    uint64_t completed, failed;
    size_t bytes_in_use;
    double link_updates; /* link-updates performed since creation */
    int preparing;       /* requests whose initial state is being built (or waits for the next tick) */
    uint64_t ticks;      /* ticks (stride steps of the running ensemble) so far */
    double prep_seconds; /* host seconds spent preparing initial states, summed over the preparer threads */
} tcym_server_info;
int tcym_server_create(tcym_ctx ctx, size_t hbm_budget_bytes, int max_active, int stride, tcym_server *out);
/* Stops the loop (running requests are abandoned) and frees everything. */
int tcym_server_destroy(tcym_server srv);
/* Queues a request (thread-safe, returns at once).  TCYM_ERR_ADMISSION if it can
 * never fit the budget. */
int tcym_server_submit(tcym_server srv, const tcym_request *req, uint64_t *id);
int tcym_server_status(tcym_server srv, uint64_t id, int *status, int *steps_done);
/* Waits up to timeout_s for the request to finish: TCYM_OK when done,
 * TCYM_ERR_TIMEOUT when the time ran out, the request's error when it failed. */
int tcym_server_wait(tcym_server srv, uint64_t id, double timeout_s);
/* N_CS series of a finished request as (steps, N_CS) pairs (up to `capacity` pairs),
 * the number of samples and the completion latency (submission to retirement). */
int tcym_server_result(tcym_server srv, uint64_t id, double *series, int capacity, int *n_samples,
                       double *latency_s);
int tcym_server_stats(tcym_server srv, tcym_server_info *out);
/* The last (up to `capacity`) ticks, oldest first: each tick's wall time in ms (the
 * ensemble's stride steps and the N_CS sample) and how many requests were being
 * prepared when it started (either array may be NULL); *n = ticks returned. */
int tcym_server_ticks(tcym_server srv, double *ms, double *preparing, int capacity, int *n);
/* One tick of the request loop. */
typedef struct {
    double ms;           /* the tick: stride steps of every running request and their N_CS samples */
    double gap_ms;       /* from the end of the previous tick to the start of this one (joins of prepared
                            requests, retirements, the ensemble's re-capture when its members changed) */
    double link_updates; /* link-updates the tick advanced */
    int active;          /* running requests */
    int preparing;       /* requests being prepared when it started */
} tcym_tick;
/* The same last (up to `capacity`) ticks as full records, oldest first. */
int tcym_server_tick_log(tcym_server srv, tcym_tick *ticks, int capacity, int *n);

#ifdef __cplusplus
}
#endif

#endif /* TCYM_H */
