/*
 * ORACLE (test infrastructure only; never part of the product).
 *
 * Compiles the reference's own real-time hot-path sources, in place, into a
 * C-callable shared library oracle/_ref/libref_su{2,3}.so.  The reference is a
 * unity build (every module is a .cpp #included into one translation unit,
 * SphaleronSimulation.cpp:13-202); this file is such a translation unit that
 * pulls in only the hot-path modules, in the reference's include order, from
 * the reference tree given by -I (see oracle/Makefile).  Nothing of the
 * reference is copied.
 *
 * Substitutions, each outside the reference's arithmetic:
 *   - <mpi.h>, "fftw3.h": empty shims (oracle/shim), the hot path calls neither.
 *   - GSL: namespace RandomNumberGenerator is supplied here, drawing Philox
 *     normals (orc_philox.h) so that the noise is the same stream the CUDA
 *     kernels draw (MISC/RNG/GSLRandomNumberGenerator.cpp is not included).
 *   - LAPACK zgeev (not vendored; reached only from MatrixILog,
 *     SUNc/SU3/AlgebraOperations.cpp:186-233, through
 *     SUNc/SU3/util/ComplexEigensystem.cpp:27-55).  When the environment
 *     variable TCYM_REF_LAPACK names a shared library that exports LAPACK's
 *     ZGEEV (as `zgeev_`, or `scipy_zgeev_` in the OpenBLAS build that SciPy
 *     ships), the call is forwarded to it unchanged: the reference then runs
 *     on a real LAPACK.  Otherwise it is restated below for what that call
 *     site asks of it, the eigenvalues and right eigenvectors of a 3x3
 *     complex matrix that is unitary there (a normal matrix): a cyclic
 *     complex Jacobi on the Hermitian (A + A^dag)/2 + g (A - A^dag)/2i, which
 *     shares A's eigenvectors, then lambda_j = v_j^dag A v_j.  MatrixILog's
 *     result, sum_j v_j (i c arg lambda_j) v_j^dag, does not depend on the
 *     eigenvectors' order or phases, so any exact eigendecomposition gives it.
 *   - The time steps Dynamics::dTau (DYNAMICS/Dynamics.cpp:17),
 *     LangevinDynamics::dTauL (DYNAMICS/LangevinDynamics.cpp:41) and
 *     ThermalDynamics::dTau (DYNAMICS/ThermalDynamics.cpp:23) are declared
 *     `static const`; `const` is defined away around those three includes so
 *     the step can be set at run time.  Each file has no other `const`.
 */
#include "Definitions.cpp"

#ifndef SU_Nc_FLAG
#error "build with -DSU_Nc_FLAG=SU2_FLAG or -DSU_Nc_FLAG=SU3_FLAG"
#endif
#define METRIC_FLAG MINKOWSKI_FLAG

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <dlfcn.h>
#include <string>

#include "SUNc/Definitions.cpp"
#include "orc_philox.h"

namespace RandomNumberGenerator {
    long int MySEED = 0;
    static uint64_t shim_seed = 0;
    static uint32_t shim_stream = 0;
    static uint64_t shim_step = 0;
    static uint64_t shim_index = 0;
    static uint64_t shim_field = 0;  /* E components of the lattice: 3 * NA * V (set by ref_init) */

    void Init(long int SEED) { MySEED = SEED; shim_seed = (uint64_t)SEED; shim_index = 0; }
    void SetStream(uint64_t seed, uint32_t stream, uint64_t step) {
        shim_seed = seed; shim_stream = stream; shim_step = step; shim_index = 0;
    }
    /* The i-th call returns the normal of E component i = a + NA*(mu + 3*site); each
     * further whole field's worth of calls (a later ReassignElectricFields, as in
     * ThermalDynamics::Thermalize) moves on to the next step of the stream. */
    DOUBLE Gauss() {
        const uint64_t na = SUNcAlgebra::VectorSize;
        uint64_t i = shim_index++;
        uint64_t round = 0;
        if (shim_field) { round = i / shim_field; i %= shim_field; }
        uint32_t a = (uint32_t)(i % na);
        uint32_t mu = (uint32_t)((i / na) % 3);
        uint32_t site = (uint32_t)(i / (3 * na));
        return orc_normal(shim_seed, shim_stream, shim_step + round, site, mu, a);
    }
    DOUBLE Gauss(DOUBLE Amplitude) { return Amplitude * Gauss(); }
    DOUBLE rng() { std::fprintf(stderr, "oracle: uniform RNG is off the hot path\n"); std::abort(); }
}

#if SU_Nc_FLAG == SU3_FLAG
// Column-major 3x3 (LAPACK's order, ComplexEigensystem.cpp:15-23): M[i + 3 j].
static void shim_jacobi_hermitian(COMPLEX H[9], COMPLEX W[9]) {
    for (int k = 0; k < 9; ++k) W[k] = COMPLEX(k % 4 == 0 ? 1.0 : 0.0, 0.0);
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 3; ++q) off += std::norm(H[p + 3 * q]);
        if (off < 1e-300) break;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 3; ++q) {
                const COMPLEX hpq = H[p + 3 * q];
                const double a = std::abs(hpq);
                if (a < 1e-300) continue;
                // G = [[c, -s e^{i phi}], [s e^{-i phi}, c]] on (p, q) zeroes (G^dag H G)_pq
                const COMPLEX e = hpq / a;
                const double tau = (H[q + 3 * q].real() - H[p + 3 * p].real()) / (2.0 * a);
                const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), sn = t * c;
                // columns: H <- H G, W <- W G
                for (int i = 0; i < 3; ++i) {
                    const COMPLEX hp = H[i + 3 * p], hq = H[i + 3 * q];
                    H[i + 3 * p] = c * hp - sn * std::conj(e) * hq;
                    H[i + 3 * q] = sn * e * hp + c * hq;
                    const COMPLEX wp = W[i + 3 * p], wq = W[i + 3 * q];
                    W[i + 3 * p] = c * wp - sn * std::conj(e) * wq;
                    W[i + 3 * q] = sn * e * wp + c * wq;
                }
                // rows: H <- G^dag H
                for (int j = 0; j < 3; ++j) {
                    const COMPLEX hp = H[p + 3 * j], hq = H[q + 3 * j];
                    H[p + 3 * j] = c * hp - sn * e * hq;
                    H[q + 3 * j] = sn * std::conj(e) * hp + c * hq;
                }
                H[p + 3 * q] = H[q + 3 * p] = COMPLEX(0.0, 0.0);
            }
    }
}
/* LAPACK's ZGEEV with gfortran's hidden CHARACTER lengths after the arguments. */
typedef void (*shim_zgeev_fn)(char const *, char const *, int *, COMPLEX *, int *, COMPLEX *, COMPLEX *, int *,
                              COMPLEX *, int *, COMPLEX *, int *, double *, int *, size_t, size_t);

/* The ZGEEV of the library TCYM_REF_LAPACK names at this call, or null (unset or empty:
 * the restatement; the library or its symbol not found: a message on stderr and the
 * restatement).  The variable is read on every call, so one process can run both. */
static shim_zgeev_fn shim_lapack_zgeev() {
    static std::string resolved_path;
    static shim_zgeev_fn fn = nullptr;
    const char *path = std::getenv("TCYM_REF_LAPACK");
    if (!path || !*path) return nullptr;
    if (resolved_path == path) return fn;
    resolved_path = path;
    fn = nullptr;
    if (void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL)) {
        fn = (shim_zgeev_fn)dlsym(h, "zgeev_");
        if (!fn) fn = (shim_zgeev_fn)dlsym(h, "scipy_zgeev_");
    }
    if (!fn) std::fprintf(stderr, "oracle: no ZGEEV in TCYM_REF_LAPACK=%s; using the restatement\n", path);
    return fn;
}

extern "C" int ref_lapack_in_use() { return shim_lapack_zgeev() != nullptr; }

extern "C" void zgeev(char const *jobvl, char const *jobvr, int *n, COMPLEX *a, int *lda, COMPLEX *w, COMPLEX *vl,
                      int *ldvl, COMPLEX *vr, int *ldvr, COMPLEX *work, int *lwork, double *rwork, int *info) {
    if (shim_zgeev_fn fn = shim_lapack_zgeev()) {
        fn(jobvl, jobvr, n, a, lda, w, vl, ldvl, vr, ldvr, work, lwork, rwork, info, 1, 1);
        return;
    }
    if (*lwork == -1) {  // workspace query
        work[0] = COMPLEX(1.0, 0.0);
        *info = 0;
        return;
    }
    if (*n != 3 || *lda != 3 || *ldvl != 3 || *ldvr != 3) {
        *info = -1;
        return;
    }
    const double g = 0.61803398874989484820;  // separates +theta from -theta
    COMPLEX H[9], W[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const COMPLEX x = a[i + 3 * j], y = std::conj(a[j + 3 * i]);
            H[i + 3 * j] = 0.5 * (x + y) + g * (x - y) / COMPLEX(0.0, 2.0);
        }
    shim_jacobi_hermitian(H, W);
    for (int j = 0; j < 3; ++j) {
        COMPLEX lam(0.0, 0.0);
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) lam += std::conj(W[i + 3 * j]) * a[i + 3 * k] * W[k + 3 * j];
        w[j] = lam;
        for (int i = 0; i < 3; ++i) vr[i + 3 * j] = vl[i + 3 * j] = W[i + 3 * j];  // normal A: left = right
    }
    *info = 0;
}
#endif

#include "IO/StringManipulation.cpp"
#include "IO/OutputManagement.cpp"
#include "LATTICE/3DGrid.cpp"
#include "LATTICE/GaugeLinks.cpp"
#include "LATTICE/ElectricFields.cpp"
#include "LATTICE/GLinksEFields.cpp"
#include "LATTICE/Indexing.cpp"
#include "CALC/Plaquettes.cpp"
#include "CALC/AvgFieldStrength.cpp"
#include "CALC/GaussViolation.cpp"
#include "CALC/ChernSimonsOperators.cpp"
#include "TOPOLOGY/ChernSimonsDerivative.cpp"
DOUBLE Qs = 1.0;
#define const
#include "DYNAMICS/Dynamics.cpp"
#undef const
#include "OBSERVABLES/BulkObservables.cpp"
#include "OBSERVABLES/GaussLawViolation.cpp"
#include "OBSERVABLES/UnitarityViolation.cpp"
#include "GAUSSLAWFIXING/GaussRestore.cpp"
#include "INITIALCONDITIONS/SetZero.cpp"
#define const
#include "DYNAMICS/ThermalDynamics.cpp"
#include "DYNAMICS/LangevinDynamics.cpp"
#undef const
#include "GRADIENTFLOW/GradientFlow.cpp"
#include "TOPOLOGY/VacuumEstimator.cpp"
#include "GRADIENTFLOW/Cooling.cpp"
#include "TOPOLOGY/CoolingMethod.cpp"
#include "IO/SaveConfiguration.cpp"

static bool g_langevin_ready = false;

extern "C" {

int ref_nc() { return Nc; }
int ref_matrix_doubles() { return (int)(SUNcGroup::MatrixSize * sizeof(SU_Nc_FUNDAMENTAL_FORMAT) / sizeof(double)); }
int ref_algebra_size() { return SUNcAlgebra::VectorSize; }

/* Lattice::N/Volume must be set before Lattice::Init (SU2Solver.cpp:106-120). */
void ref_init(int nx, int ny, int nz) {
    if (GLinks::U) { delete GLinks::U; delete EFields::E; }
    Lattice::N[0] = nx; Lattice::N[1] = ny; Lattice::N[2] = nz;
    Lattice::Volume = nx * ny * nz;
    RandomNumberGenerator::shim_field = 3ull * SUNcAlgebra::VectorSize * (uint64_t)Lattice::Volume;
    Lattice::Init();
    Dynamics::Reset();
    LangevinDynamics::Reset();
    GradientFlow::Reset();
    if (g_langevin_ready) { delete LangevinVariables::Xi; g_langevin_ready = false; }
}

void ref_set(const double *U, const double *E) {
    std::memcpy(GLinks::U->U, U, sizeof(SU_Nc_FUNDAMENTAL_FORMAT) * 3 * SUNcGroup::MatrixSize * GLinks::U->Volume);
    std::memcpy(EFields::E->E, E, sizeof(double) * 3 * SUNcAlgebra::VectorSize * EFields::E->Volume);
}

void ref_get(double *U, double *E) {
    std::memcpy(U, GLinks::U->U, sizeof(SU_Nc_FUNDAMENTAL_FORMAT) * 3 * SUNcGroup::MatrixSize * GLinks::U->Volume);
    std::memcpy(E, EFields::E->E, sizeof(double) * 3 * SUNcAlgebra::VectorSize * EFields::E->Volume);
}

void ref_set_zero() { InitialConditions::SetZero(0, Lattice::N[0] - 1, 0, Lattice::N[1] - 1, 0, Lattice::N[2] - 1); }

/* Dynamics::Update (DYNAMICS/Dynamics.cpp:204-218), nsteps times at time step dt. */
void ref_leapfrog(double dt, int nsteps) {
    Dynamics::dTau = dt;
    for (int s = 0; s < nsteps; ++s) Dynamics::Update(GLinks::U, EFields::E);
}

/* E half-kick only (Dynamics.cpp:145-197), for unit parity of the force. */
void ref_update_e(double dt) {
    Dynamics::dTau = dt;
    Dynamics::SetMetric();
    Dynamics::UpdateElectricFields(0, Lattice::N[0] - 1, 0, Lattice::N[1] - 1, 0, Lattice::N[2] - 1, GLinks::U, EFields::E);
}

/* Link update only (Dynamics.cpp:97-138). */
void ref_update_u(double dt) {
    Dynamics::dTau = dt;
    Dynamics::SetMetric();
    Dynamics::UpdateGaugeLinks(0, Lattice::N[0] - 1, 0, Lattice::N[1] - 1, 0, Lattice::N[2] - 1, GLinks::U, EFields::E);
}

/* LangevinDynamics::UpdateRandomGaussianNoise + UpdateFields
 * (DYNAMICS/LangevinDynamics.cpp:260-311); beta = 1/T (LangevinDynamics.cpp:23). */
void ref_langevin(double dt, double T, uint64_t seed, uint64_t step0, int nsteps) {
    if (!g_langevin_ready) { LangevinVariables::Init(); g_langevin_ready = true; }
    LangevinDynamics::dTauL = dt;
    LangevinDynamics::beta = 1.0 / T;
    for (int s = 0; s < nsteps; ++s) {
        RandomNumberGenerator::SetStream(seed, ORC_STREAM_NOISE, step0 + (uint64_t)s);
        LangevinDynamics::UpdateRandomGaussianNoise();
        LangevinDynamics::UpdateFields(GLinks::U, EFields::E);
    }
}

/* GradientFlow::StandardUpdate / CalibrationUpdate (GRADIENTFLOW/GradientFlow.cpp:150-188).
 * Returns ChernSimonsNumber::DeltaNCsCooling accumulated over the calibrated steps. */
double ref_flow(double sqrt_dctau_over_a, int nsteps, int calibrate) {
    GradientFlow::SqrtDcTauOverSpacing = sqrt_dctau_over_a;
    GradientFlow::Reset();
    ChernSimonsNumber::DeltaNCsCooling = 0.0;
    for (int s = 0; s < nsteps; ++s) {
        if (calibrate) GradientFlow::CalibrationUpdate(GLinks::U, EFields::E);
        else GradientFlow::StandardUpdate(GLinks::U, EFields::E);
    }
    return ChernSimonsNumber::DeltaNCsCooling;
}

/* GaussLawRestoration::Restore (GAUSSLAWFIXING/GaussRestore.cpp:131-167). */
void ref_gauss_restore() { GaussLawRestoration::Restore(GLinks::U, EFields::E); }

/* ThermalDynamics::ReassignElectricFields (DYNAMICS/ThermalDynamics.cpp:205-226):
 * E = N(0,1)/sqrt(beta) from the Philox field stream, then Gauss restore. */
void ref_thermal_efield(double beta, uint64_t seed) {
    ThermalDynamics::beta = beta;
    RandomNumberGenerator::SetStream(seed, ORC_STREAM_EFIELD, 0);
    ThermalDynamics::ReassignElectricFields();
}

/* ThermalDynamics::Thermalize(rounds, max_time) (DYNAMICS/ThermalDynamics.cpp:260-314)
 * with ThermalDynamics::dTau = dtau, writing its energy series to
 * <outdir>/ThermalEnergyID<seed>.txt as the reference does. */
void ref_thermalize(double beta, uint64_t seed, int rounds, double max_time, double dtau, const char *outdir) {
    IO::OutputDirectory = StringManipulation::StringCast(outdir, "/");
    ThermalDynamics::beta = beta;
    ThermalDynamics::dTau = dtau;
    ThermalDynamics::Reset();
    RandomNumberGenerator::MySEED = (long int)seed;
    RandomNumberGenerator::SetStream(seed, ORC_STREAM_EFIELD, 0);
    ThermalDynamics::Thermalize(rounds, max_time);
}

/* ChernSimonsNumber::CoolingMethod (TOPOLOGY/CoolingMethod.cpp): Init with the
 * given standard blocking level, cooling steps, Cooling::BlockFrequency and flow
 * step, then Start (:124-135) or Update(measure) (:141-166) on the current links;
 * update returns ChernSimonsNumber::DeltaNCsCoolRealTime.  SU(3) measurements reach
 * MatrixILog, i.e. the zgeev stub, and abort: SU(2) only for measure = 1. */
void ref_cooling_init(int blocking, int max_steps, int block_frequency, double sqrt_dctau) {
    ChernSimonsNumber::CoolingMethod::StandardBlockingLevel = blocking;
    ChernSimonsNumber::CoolingMethod::StandardCoolingMaxSteps = max_steps;
    Cooling::BlockFrequency = block_frequency;
    GradientFlow::SqrtDcTauOverSpacing = sqrt_dctau;
    ChernSimonsNumber::DeltaNCsCoolRealTime = 0.0;
    ChernSimonsNumber::CoolingMethod::Init();
}
void ref_cooling_start() { ChernSimonsNumber::CoolingMethod::Start(); }
double ref_cooling_update(int measure) {
    ChernSimonsNumber::CoolingMethod::Update(measure);
    return ChernSimonsNumber::DeltaNCsCoolRealTime;
}
/* the cooled links UOld (after Start/Update it equals UNew) */
void ref_cooling_links(double *U) {
    GaugeLinks *u = ChernSimonsNumber::CoolingMethod::UOld;
    std::memcpy(U, u->U, sizeof(SU_Nc_FUNDAMENTAL_FORMAT) * 3 * SUNcGroup::MatrixSize * u->Volume);
}
/* SUNcAlgebra::Operations::MatrixILog (SU2/AlgebraOperations.cpp:56-74) */
void ref_matrix_ilog(double c, const double *v, double *out) {
    SU_Nc_FUNDAMENTAL_FORMAT m[SUNcGroup::MatrixSize];
    std::memcpy(m, v, sizeof(m));
    SUNcAlgebra::Operations::MatrixILog(c, m, out);
}

/* IO::SaveConfiguration (IO/SaveConfiguration.cpp:3-56): writes
 * <outdir>/<ufname>ID<seed>.txt and <outdir>/<efname>ID<seed>.txt. */
void ref_save_configuration(const char *outdir, const char *ufname, const char *efname, uint64_t seed) {
    IO::OutputDirectory = StringManipulation::StringCast(outdir, "/");
    RandomNumberGenerator::MySEED = (long int)seed;
    IO::SaveConfiguration(ufname, efname);
}

/* Observables: Bulk (OBSERVABLES/BulkObservables.cpp:133-143), GaussLaw
 * (GaussLawViolation.cpp:13-61), Unitarity (UnitarityViolation.cpp:13-51), and
 * both E.B operators (CALC/ChernSimonsOperators.cpp:4-47, 72-382).
 * out[0..14] = T00, ELECTRIC, MAGNETIC, ESqr[3], BSqr[3], gauss signed max,
 * gauss rms, unitarity max, unitarity rms, clover E.B, improved E.B. */
void ref_observables(double *out) {
    Dynamics::SetMetric();
    GaugeLinks *U = GLinks::U;
    ElectricFields *E = EFields::E;
    Observables::Bulk::Update(U, E);
    out[0] = Observables::Bulk::T00();
    out[1] = Observables::Bulk::ELECTRIC();
    out[2] = Observables::Bulk::MAGNETIC();
    for (int i = 0; i < 3; ++i) { out[3 + i] = Observables::Bulk::ESqr[i]; out[6 + i] = Observables::Bulk::BSqr[i]; }
    Observables::GaussLaw::UpdateViolation(0, U->N[0] - 1, 0, U->N[1] - 1, 0, U->N[2] - 1, U, E);
    out[9] = Observables::GaussLaw::GlobalMaxViolation;
    out[10] = Observables::GaussLaw::GlobalAvgViolation;
    Observables::Unitarity::UpdateViolation(0, U->N[0] - 1, 0, U->N[1] - 1, 0, U->N[2] - 1, U);
    out[11] = Observables::Unitarity::GlobalMaxViolation;
    out[12] = Observables::Unitarity::GlobalAvgViolation;
    out[13] = UnimprovedOperators::ComputeEDotB(U, E);
    out[14] = ImprovedOperators::ComputeEDotB(U, E);
}

/* Group kernels for unit tests of the device math. */
void ref_matrix_iexp(double c, const double *alpha, double *out) {
    SUNcAlgebra::Operations::MatrixIExp(c, (DOUBLE *)alpha, (SU_Nc_FUNDAMENTAL_FORMAT *)out);
}
void ref_retr_igen(const double *V, double *out) {
    SUNcGroup::Operations::ReTrIGenU((SU_Nc_FUNDAMENTAL_FORMAT *)V, out);
}
void ref_inverse_adjoint(const double *V, const double *A, double *out) {
    SUNcAlgebra::Operations::InverseAdjointMultiplication((SU_Nc_FUNDAMENTAL_FORMAT *)V, (DOUBLE *)A, out);
}
void ref_adjoint(const double *V, const double *A, double *out) {
    SUNcAlgebra::Operations::AdjointMultiplication((SU_Nc_FUNDAMENTAL_FORMAT *)V, (DOUBLE *)A, out);
}

}  // extern "C"
