// tcym_compat.hpp — the reference's C++ hot-path API over the tcym C ABI.
//
// Header-only.  A driver written against markmace/TopologicalCYMSolver's
// real-time path (GaugeLinks, ElectricFields, Dynamics, LangevinDynamics,
// GradientFlow, Cooling, GaussLawRestoration, Observables, the E.B operators and
// ChernSimonsNumber::NCsDot) includes this header instead of those modules and
// links libtcym.so.  The gauge group is fixed at compile time as in the
// reference (SUNc/Definitions.cpp:22-49): define TCYM_NC to 2 or 3 (default 3)
// before including.  TCYM_COMPAT_PRECISION selects TCYM_FP64 (default, the
// plain drop-in) or TCYM_FP32 storage.
//
// Memory model.  GaugeLinks::U and ElectricFields::E are host arrays in the
// reference's layouts (LATTICE/GaugeLinks.cpp:27-47, LATTICE/ElectricFields.cpp:36-46).
// The first hot-path call on a (links, fields) pair binds it to one device
// lattice; the device copy then holds the state.  Get() (or Host()) brings the
// host array up to date and marks it as possibly written by the caller, so the
// next hot-path call uploads it again.  Only whole-lattice ranges are
// accepted where the reference takes xLow..zHigh bounds.
//
// Failures of the library throw std::runtime_error with tcym_last_error().
#pragma once

#include <cmath>
#include <complex>
#include <fstream>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "tcym.h"

#ifndef TCYM_NC
#define TCYM_NC 3
#endif
#ifndef TCYM_COMPAT_PRECISION
#define TCYM_COMPAT_PRECISION TCYM_FP64
#endif
#ifndef TCYM_COMPAT_DEVICE
#define TCYM_COMPAT_DEVICE 0
#endif

typedef int INT;
typedef double DOUBLE;
typedef std::complex<DOUBLE> COMPLEX;
#if TCYM_NC == 2
typedef DOUBLE SU_Nc_FUNDAMENTAL_FORMAT;
#else
typedef COMPLEX SU_Nc_FUNDAMENTAL_FORMAT;
#endif
typedef DOUBLE SU_Nc_ALGEBRA_FORMAT;

namespace SUNcGroup {
static const int MatrixSize = TCYM_NC == 2 ? 4 : 9;  // elements of SU_Nc_FUNDAMENTAL_FORMAT per link
}
namespace SUNcAlgebra {
static const int VectorSize = TCYM_NC == 2 ? 3 : 8;
}

class GaugeLinks;
class ElectricFields;

namespace tcym_compat {

inline tcym_ctx &context() {
    static tcym_ctx ctx = nullptr;
    if (!ctx) {
        int rc = tcym_ctx_create(TCYM_COMPAT_DEVICE, &ctx);
        if (rc != TCYM_OK) throw std::runtime_error("tcym: cannot open the CUDA device (code " + std::to_string(rc) + ")");
    }
    return ctx;
}

inline void check(int rc, const char *what) {
    if (rc != TCYM_OK)
        throw std::runtime_error(std::string("tcym: ") + what + " failed (code " + std::to_string(rc) +
                                 "): " + tcym_last_error(context()));
}

// where the newest copy of one object lives
enum class Fresh { Host, Device };

// device lattice bound to one (links, fields) pair
struct Binding {
    tcym_lattice lat = nullptr;
    GaugeLinks *U = nullptr;
    ElectricFields *E = nullptr;
};

inline void unbind(Binding *b);

}  // namespace tcym_compat

class GaugeLinks {
   public:
    INT Volume;
    const static INT Dimension = 3;
    DOUBLE a[Dimension];
    DOUBLE aCube;
    INT N[Dimension];
    SU_Nc_FUNDAMENTAL_FORMAT *U;

    tcym_compat::Binding *binding = nullptr;
    tcym_compat::Fresh fresh = tcym_compat::Fresh::Host;

    GaugeLinks(INT Nx, INT Ny, INT Nz, INT ax, INT ay, INT az) {
        Volume = Nx * Ny * Nz;
        N[0] = Nx; N[1] = Ny; N[2] = Nz;
        a[0] = ax; a[1] = ay; a[2] = az;
        aCube = a[0] * a[1] * a[2];
        U = new SU_Nc_FUNDAMENTAL_FORMAT[Dimension * SUNcGroup::MatrixSize * Volume]();
    }
    ~GaugeLinks();
    GaugeLinks(const GaugeLinks &) = delete;
    GaugeLinks &operator=(const GaugeLinks &) = delete;

    INT Index3D(INT x, INT y, INT z) const {
        auto m = [](INT v, INT n) { return v >= 0 ? v % n : (v % n + n) % n; };
        return m(x, N[0]) + N[0] * (m(y, N[1]) + N[1] * m(z, N[2]));
    }
    INT Index(INT x, INT y, INT z, INT mu) const { return SUNcGroup::MatrixSize * (mu + Dimension * Index3D(x, y, z)); }
    void GetPosition(INT Index, INT &x, INT &y, INT &z) const {
        z = Index / (N[0] * N[1]);
        y = (Index - z * (N[0] * N[1])) / (N[0]);
        x = (Index - N[0] * (y + N[1] * z));
    }
    // host array, brought up to date; the caller may write it
    SU_Nc_FUNDAMENTAL_FORMAT *Host();
    SU_Nc_FUNDAMENTAL_FORMAT *Get(INT x, INT y, INT z, INT mu) { return &(Host()[Index(x, y, z, mu)]); }
    void SetIdentity() {
        SU_Nc_FUNDAMENTAL_FORMAT *h = Host();
        for (INT s = 0; s < Dimension * Volume; ++s)
            for (int k = 0; k < SUNcGroup::MatrixSize; ++k) {
#if TCYM_NC == 2
                h[SUNcGroup::MatrixSize * s + k] = k == 3 ? 1.0 : 0.0;
#else
                h[SUNcGroup::MatrixSize * s + k] = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
#endif
            }
    }
};

class ElectricFields {
   public:
    INT Volume;
    const static INT Dimension = 3;
    DOUBLE a[Dimension];
    DOUBLE aCube;
    INT N[Dimension];
    SU_Nc_ALGEBRA_FORMAT *E;

    tcym_compat::Binding *binding = nullptr;
    tcym_compat::Fresh fresh = tcym_compat::Fresh::Host;

    ElectricFields(INT Nx, INT Ny, INT Nz, INT ax, INT ay, INT az) {
        Volume = Nx * Ny * Nz;
        N[0] = Nx; N[1] = Ny; N[2] = Nz;
        a[0] = ax; a[1] = ay; a[2] = az;
        aCube = a[0] * a[1] * a[2];
        E = new SU_Nc_ALGEBRA_FORMAT[Dimension * SUNcAlgebra::VectorSize * Volume]();
    }
    ~ElectricFields();
    ElectricFields(const ElectricFields &) = delete;
    ElectricFields &operator=(const ElectricFields &) = delete;

    INT Index3D(INT x, INT y, INT z) const {
        auto m = [](INT v, INT n) { return v >= 0 ? v % n : (v % n + n) % n; };
        return m(x, N[0]) + N[0] * (m(y, N[1]) + N[1] * m(z, N[2]));
    }
    INT Index(INT x, INT y, INT z, INT mu, INT a) const {
        return a + SUNcAlgebra::VectorSize * (mu + Dimension * Index3D(x, y, z));
    }
    SU_Nc_ALGEBRA_FORMAT *Host();
    SU_Nc_ALGEBRA_FORMAT *Get(INT x, INT y, INT z, INT mu, INT a) { return &(Host()[Index(x, y, z, mu, a)]); }
    void SetZero() {
        std::memset(Host(), 0, sizeof(SU_Nc_ALGEBRA_FORMAT) * Dimension * SUNcAlgebra::VectorSize * Volume);
    }
};

namespace tcym_compat {

// Pulls the newest copy to the host (no-op when the host is newest).
inline void pull(GaugeLinks *U) {
    if (U->binding && U->fresh == Fresh::Device)
        check(tcym_lattice_download(U->binding->lat, reinterpret_cast<double *>(U->U), nullptr), "download links");
    U->fresh = Fresh::Host;
}
inline void pull(ElectricFields *E) {
    if (E->binding && E->fresh == Fresh::Device)
        check(tcym_lattice_download(E->binding->lat, nullptr, E->E), "download fields");
    E->fresh = Fresh::Host;
}

inline void unbind(Binding *b) {
    if (!b) return;
    if (b->U) { pull(b->U); b->U->binding = nullptr; }
    if (b->E) { pull(b->E); b->E->binding = nullptr; }
    tcym_lattice_destroy(b->lat);
    delete b;
}

// Binds (U, E) to one device lattice (E may be null for link-only calls) and
// uploads whatever the host holds newer.  Returns the lattice.
inline tcym_lattice bind(GaugeLinks *U, ElectricFields *E) {
    if (!U) throw std::invalid_argument("tcym: null GaugeLinks");
    Binding *b = U->binding;
    if (!b || (E && b->E != E)) {
        if (b) unbind(b);
        if (E && E->binding) unbind(E->binding);
        b = new Binding();
        const double a[3] = {U->a[0], U->a[1], U->a[2]};
        check(tcym_lattice_create_ex(context(), TCYM_NC, U->N[0], U->N[1], U->N[2], a, TCYM_COMPAT_PRECISION, &b->lat),
              "lattice create");
        b->U = U;
        U->binding = b;
        U->fresh = Fresh::Host;
        if (E) {
            b->E = E;
            E->binding = b;
            E->fresh = Fresh::Host;
        } else {
            check(tcym_set_zero(b->lat), "set zero");  // fields of a link-only binding start at zero
            check(tcym_lattice_upload(b->lat, reinterpret_cast<const double *>(U->U), nullptr), "upload links");
            U->fresh = Fresh::Device;
        }
    }
    if (U->fresh == Fresh::Host)
        check(tcym_lattice_upload(b->lat, reinterpret_cast<const double *>(U->U), nullptr), "upload links");
    if (E && E->fresh == Fresh::Host) check(tcym_lattice_upload(b->lat, nullptr, E->E), "upload fields");
    U->fresh = Fresh::Device;
    if (E) E->fresh = Fresh::Device;
    return b->lat;
}

inline void whole(const GaugeLinks *U, INT xl, INT xh, INT yl, INT yh, INT zl, INT zh) {
    if (xl != 0 || yl != 0 || zl != 0 || xh != U->N[0] - 1 || yh != U->N[1] - 1 || zh != U->N[2] - 1)
        throw std::invalid_argument("tcym: only whole-lattice ranges are supported");
}

inline tcym_obs observables(GaugeLinks *U, ElectricFields *E) {
    tcym_obs o;
    int rc = tcym_observables(bind(U, E), &o);
    if (rc != TCYM_OK && rc != TCYM_ERR_NONFINITE) check(rc, "observables");
    return o;
}

}  // namespace tcym_compat

inline SU_Nc_FUNDAMENTAL_FORMAT *GaugeLinks::Host() {
    tcym_compat::pull(this);
    return U;
}
inline GaugeLinks::~GaugeLinks() {
    if (binding) {
        binding->U = nullptr;
        tcym_compat::unbind(binding);
    }
    delete[] U;
}
inline SU_Nc_ALGEBRA_FORMAT *ElectricFields::Host() {
    tcym_compat::pull(this);
    return E;
}
inline ElectricFields::~ElectricFields() {
    if (binding) {
        binding->E = nullptr;
        tcym_compat::unbind(binding);
    }
    delete[] E;
}

// Copy(UCopy, UOriginal) / Copy(ECopy, EOriginal) (LATTICE/GaugeLinks.cpp:91-107, ElectricFields.cpp:90-104)
inline void Copy(GaugeLinks *UCopy, GaugeLinks *UOriginal) {
    std::memcpy(UCopy->Host(), UOriginal->Host(),
                sizeof(SU_Nc_FUNDAMENTAL_FORMAT) * 3 * SUNcGroup::MatrixSize * UOriginal->Volume);
}
inline void Copy(ElectricFields *ECopy, ElectricFields *EOriginal) {
    std::memcpy(ECopy->Host(), EOriginal->Host(), sizeof(DOUBLE) * 3 * SUNcAlgebra::VectorSize * EOriginal->Volume);
}

// ------------------------------------------------------------ globals
namespace Lattice {
static const int Dimension = 3;
inline INT N[3] = {64, 64, 64};
static const DOUBLE a[3] = {1.0, 1.0, 1.0};
inline DOUBLE aScale = 1.0;
inline INT Volume = 64 * 64 * 64;
inline DOUBLE aCube = 1.0;
}  // namespace Lattice
namespace GLinks {
inline GaugeLinks *U = nullptr;
}
namespace EFields {
inline ElectricFields *E = nullptr;
}
namespace Lattice {
// Lattice::Init (LATTICE/GLinksEFields.cpp:36-45)
inline void Init() {
    GLinks::U = new GaugeLinks(N[0], N[1], N[2], (INT)a[0], (INT)a[1], (INT)a[2]);
    EFields::E = new ElectricFields(N[0], N[1], N[2], (INT)a[0], (INT)a[1], (INT)a[2]);
    aCube = GLinks::U->a[0] * GLinks::U->a[1] * GLinks::U->a[2];
}
}  // namespace Lattice

// ------------------------------------------------------------ dynamics
namespace Dynamics {
inline DOUBLE dTau = 0.025;  // a run-time value here (static const in DYNAMICS/Dynamics.cpp:17)
inline INT tSteps = 0;
inline DOUBLE Time() { return tSteps * dTau; }
inline void Reset() { tSteps = 0; }
inline void SetMetric() {}
inline void UpdateElectricFields(INT xl, INT xh, INT yl, INT yh, INT zl, INT zh, GaugeLinks *U, ElectricFields *E) {
    tcym_compat::whole(U, xl, xh, yl, yh, zl, zh);
    tcym_compat::check(tcym_update_e(tcym_compat::bind(U, E), dTau), "update E");
}
inline void UpdateGaugeLinks(INT xl, INT xh, INT yl, INT yh, INT zl, INT zh, GaugeLinks *U, ElectricFields *E) {
    tcym_compat::whole(U, xl, xh, yl, yh, zl, zh);
    tcym_compat::check(tcym_update_u(tcym_compat::bind(U, E), dTau), "update U");
}
// Dynamics::Update (DYNAMICS/Dynamics.cpp:204-218)
inline void Update(GaugeLinks *U, ElectricFields *E) {
    tcym_compat::check(tcym_leapfrog(tcym_compat::bind(U, E), dTau, 1), "leapfrog");
    ++tSteps;
}
inline void Update() { Update(GLinks::U, EFields::E); }
}  // namespace Dynamics

namespace RandomNumberGenerator {
inline long int MySEED = 0;  // seeds the Philox streams of the compat layer
}

namespace IO {
inline std::string OutputDirectory;  // with a trailing '/', as IO/OutputManagement.cpp sets it
inline std::string InputDirectory, InputUFile, InputEFile;
}

namespace ThermalDynamics {
inline DOUBLE beta = 2.0;
inline DOUBLE dTau = 0.0375;  // static const in DYNAMICS/ThermalDynamics.cpp:23
}

namespace GaussLawRestoration {
inline DOUBLE GlobalMaxViolation = 0.0;
inline DOUBLE GlobalAvgViolation = 0.0;
// GaussLawRestoration::Restore (GAUSSLAWFIXING/GaussRestore.cpp:131-167)
inline void Restore(GaugeLinks *U, ElectricFields *E) {
    int it = 0;
    double mx = 0.0;
    tcym_compat::check(tcym_gauss_restore(tcym_compat::bind(U, E), 1e-14, 10000, &it, &mx), "Gauss restore");
    GlobalMaxViolation = mx;
    std::cerr << "#GAUSS LAW FIXING " << it << " ITERATIONS, MAX " << mx << std::endl;
}
inline void Restore() { Restore(GLinks::U, EFields::E); }
}  // namespace GaussLawRestoration

namespace ThermalDynamics {
// ReassignElectricFields (DYNAMICS/ThermalDynamics.cpp:205-226): E = N(0,1)/sqrt(beta), then restore
inline void ReassignElectricFields() {
    tcym_lattice lat = tcym_compat::bind(GLinks::U, EFields::E);
    tcym_compat::check(tcym_gaussian_efield(lat, 1.0 / std::sqrt(beta), (uint64_t)RandomNumberGenerator::MySEED),
                       "Gaussian fields");
    GaussLawRestoration::Restore(GLinks::U, EFields::E);
}
// Thermalize(MaxSteps, MaxTime) (DYNAMICS/ThermalDynamics.cpp:260-314), writing the
// energy series to <OutputDirectory>ThermalEnergyID<seed>.txt as the reference does
inline void Thermalize(INT MaxSteps, DOUBLE MaxTime) {
    long steps = 0;
    while ((double)steps * dTau < MaxTime) ++steps;
    std::vector<double> series(7 * (size_t)MaxSteps * (size_t)(steps / 20 + 1));
    int n = 0;
    tcym_compat::check(tcym_thermalize(tcym_compat::bind(GLinks::U, EFields::E), beta,
                                       (uint64_t)RandomNumberGenerator::MySEED, (int)MaxSteps, MaxTime, dTau, 0.0,
                                       20, series.data(), (int)(series.size() / 7), &n),
                       "thermalize");
    std::ofstream out(IO::OutputDirectory + "ThermalEnergyID" + std::to_string(RandomNumberGenerator::MySEED) +
                      ".txt");
    out.precision(15);
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < 7; ++k) out << (k ? " " : "") << series[7 * (size_t)i + k];
        out << "\n";
    }
}
}  // namespace ThermalDynamics

namespace InitialConditions {
// InitialConditions::SetZero (INITIALCONDITIONS/SetZero.cpp:3-24)
inline void SetZero() {
    tcym_compat::check(tcym_set_zero(tcym_compat::bind(GLinks::U, EFields::E)), "set zero");
}
}  // namespace InitialConditions

namespace LangevinDynamics {
inline DOUBLE beta = 2.0;
inline DOUBLE dTauL = 0.001;  // static const in DYNAMICS/LangevinDynamics.cpp:41
inline INT tauLSteps = 0;
inline DOUBLE Time() { return tauLSteps * dTauL; }
inline void Reset() { tauLSteps = 0; }
// The noise xi is drawn inside the step from the Philox stream (MySEED, step, site, mu, a);
// there is no noise array to refill (UpdateRandomGaussianNoise, LangevinDynamics.cpp:260-286).
inline void UpdateRandomGaussianNoise() {}
// LangevinDynamics::UpdateFields (LangevinDynamics.cpp:300-311), damping 1 as the reference
inline void UpdateFields(GaugeLinks *U, ElectricFields *E) {
    tcym_compat::check(tcym_langevin(tcym_compat::bind(U, E), dTauL, 1.0, 1.0 / beta,
                                     (uint64_t)RandomNumberGenerator::MySEED, (uint64_t)tauLSteps, 1),
                       "Langevin step");
    ++tauLSteps;
}
inline void UpdateFields() { UpdateFields(GLinks::U, EFields::E); }
inline void Update() { UpdateFields(); }
}  // namespace LangevinDynamics

namespace UnimprovedOperators {
// clover E.B (CALC/ChernSimonsOperators.cpp:4-47)
inline DOUBLE ComputeEDotB(GaugeLinks *U, ElectricFields *E) {
    double v = 0.0;
    tcym_compat::check(tcym_edotb(tcym_compat::bind(U, E), &v), "clover E.B");
    return v;
}
}  // namespace UnimprovedOperators

namespace ImprovedOperators {
// O(a^2)-improved E.B (CALC/ChernSimonsOperators.cpp:72-382)
inline DOUBLE ComputeEDotB(GaugeLinks *U, ElectricFields *E) {
    double v = 0.0;
    tcym_compat::check(tcym_edotb_improved(tcym_compat::bind(U, E), &v), "improved E.B");
    return v;
}
}  // namespace ImprovedOperators

namespace ChernSimonsNumber {
inline DOUBLE DeltaNCsRealTime = 0.0;
inline DOUBLE DeltaNCsCooling = 0.0;
// NCsDot (TOPOLOGY/ChernSimonsDerivative.cpp:31-49): improved operator, 1/(8 pi^2)
inline DOUBLE NCsDot(GaugeLinks *U, ElectricFields *E) {
    return 0.125 * ImprovedOperators::ComputeEDotB(U, E) / (3.14159265358979323846 * 3.14159265358979323846);
}
}  // namespace ChernSimonsNumber

namespace GradientFlow {
inline DOUBLE cTau = 0.0;
inline INT CoolingSteps = 0;
inline DOUBLE SqrtDcTauOverSpacing = 0.5 / 1.414213562373095048801688724209698;
inline void Reset() { cTau = 0.0; CoolingSteps = 0; }
inline DOUBLE CoolingTime() { return cTau; }
inline DOUBLE DcTau(GaugeLinks *U) { return SqrtDcTauOverSpacing * SqrtDcTauOverSpacing * std::pow(U->aCube, 2.0 / 3.0); }
// StandardUpdate (GRADIENTFLOW/GradientFlow.cpp:150-165)
inline void StandardUpdate(GaugeLinks *U, ElectricFields *E) {
    const double d = DcTau(U);
    tcym_compat::check(tcym_flow(tcym_compat::bind(U, E), d, 1, TCYM_FLOW_SIMULTANEOUS, 0, nullptr), "flow");
    ++CoolingSteps;
    cTau += d;
}
// CalibrationUpdate (GradientFlow.cpp:168-188)
inline void CalibrationUpdate(GaugeLinks *U, ElectricFields *E) {
    const double d = DcTau(U);
    double dn = 0.0;
    tcym_compat::check(tcym_flow(tcym_compat::bind(U, E), d, 1, TCYM_FLOW_SIMULTANEOUS, TCYM_NCS_IMPROVED, &dn),
                       "calibrated flow");
    ChernSimonsNumber::DeltaNCsCooling += dn;
    ++CoolingSteps;
    cTau += d;
}
}  // namespace GradientFlow

// Block(GaugeLinks**) (LATTICE/GaugeLinks.cpp:124-145): the links replaced by the
// blocked ones, U'_mu(x) = U_mu(2x) U_mu(2x + mu), on half the extents and twice
// the spacings (computed on the device, tcym_lattice_block)
inline void Block(GaugeLinks **UOld) {
    GaugeLinks *u = *UOld;
    GaugeLinks *n = new GaugeLinks(u->N[0] / 2, u->N[1] / 2, u->N[2] / 2, (INT)(2 * u->a[0]), (INT)(2 * u->a[1]),
                                   (INT)(2 * u->a[2]));
    tcym_lattice src = tcym_compat::bind(u, nullptr);
    tcym_compat::check(tcym_lattice_block(src, tcym_compat::bind(n, nullptr)), "block links");
    n->fresh = tcym_compat::Fresh::Device;
    delete u;
    *UOld = n;
}
// Block(ElectricFields**) (LATTICE/ElectricFields.cpp:113-127): zero fields on half the extents
inline void Block(ElectricFields **EOld) {
    ElectricFields *e = *EOld;
    ElectricFields *n = new ElectricFields(e->N[0] / 2, e->N[1] / 2, e->N[2] / 2, (INT)(2 * e->a[0]),
                                           (INT)(2 * e->a[1]), (INT)(2 * e->a[2]));
    n->SetZero();
    delete e;
    *EOld = n;
}

namespace Cooling {
inline INT BlockFrequency = 0;
// CoolNSave (GRADIENTFLOW/Cooling.cpp:156-179) with Perform's blocking (:69-143):
// flow a copy of UHot from E = 0 for MaxCoolingSteps steps, blocking links and
// fields after each step that is a multiple of BlockFrequency 8^b while fewer than
// MaxBlockingNumber Blocks were made; the result goes to UCold (of the blocked size).
inline void CoolNSave(std::string, DOUBLE MaxCoolingSteps, INT MaxBlockingNumber, GaugeLinks *UHot, GaugeLinks *UCold) {
    GaugeLinks *U = new GaugeLinks(UHot->N[0], UHot->N[1], UHot->N[2], (INT)UHot->a[0], (INT)UHot->a[1], (INT)UHot->a[2]);
    ElectricFields *E =
        new ElectricFields(UHot->N[0], UHot->N[1], UHot->N[2], (INT)UHot->a[0], (INT)UHot->a[1], (INT)UHot->a[2]);
    Copy(U, UHot);
    E->SetZero();
    GradientFlow::Reset();
    INT blocking = 0;
    while (GradientFlow::CoolingSteps < MaxCoolingSteps) {
        GradientFlow::StandardUpdate(U, E);
        if (blocking < MaxBlockingNumber && BlockFrequency > 0 &&
            GradientFlow::CoolingSteps % (BlockFrequency * (INT)std::pow(8, blocking)) == 0) {
            ::Block(&U);
            ::Block(&E);
            ++blocking;
        }
    }
    if (UCold->Volume != U->Volume) {
        delete U;
        delete E;
        throw std::invalid_argument("tcym: CoolNSave: UCold does not have the blocked extents");
    }
    Copy(UCold, U);
    delete U;
    delete E;
}
}  // namespace Cooling

namespace ChernSimonsNumber {
inline DOUBLE DeltaNCsCoolRealTime = 0.0;
// CoolingMethod (TOPOLOGY/CoolingMethod.cpp) on GLinks::U at StandardBlockingLevel
// (the reference's drivers use 0, SphaleronSimulation.cpp:236) with Cooling::BlockFrequency;
// the cooled copies live on the device (tcym_cooling_*), flowed with
// GradientFlow::SqrtDcTauOverSpacing.
namespace CoolingMethod {
inline INT StandardBlockingLevel = 0;
inline INT StandardCoolingMaxSteps = 128;
inline tcym_cooling state = nullptr;
// Init (:19-32)
inline void Init() {
    if (state) tcym_cooling_destroy(state);
    state = nullptr;
    tcym_compat::check(tcym_cooling_create_ex(tcym_compat::bind(GLinks::U, EFields::E), (int)StandardCoolingMaxSteps,
                                              GradientFlow::SqrtDcTauOverSpacing, (int)StandardBlockingLevel,
                                              (int)Cooling::BlockFrequency, &state),
                       "cooling init");
}
// Start (:124-135)
inline void Start() { tcym_compat::check(tcym_cooling_start(state), "cooling start"); }
// Update(Measure) (:141-166): DeltaNCsCoolRealTime += GetDeltaNCs(1) when measuring
inline void Update(INT Measure) {
    tcym_compat::bind(GLinks::U, EFields::E);  // the host mirror, if dirty, to the device first
    double d = 0.0;
    tcym_compat::check(tcym_cooling_update(state, (int)Measure, &d), "cooling update");
    DeltaNCsCooling = 0.0;
    if (Measure == 1) DeltaNCsCoolRealTime += d;
}
// GetDeltaNCs(NOrder) (:77-120) on the current pair of cooled configurations
inline DOUBLE GetDeltaNCs(INT NOrder) {
    double d = 0.0;
    tcym_compat::check(tcym_cooling_delta_ncs(state, (int)NOrder, &d), "cooled delta N_CS");
    return d;
}
}  // namespace CoolingMethod
}  // namespace ChernSimonsNumber

namespace IO {
// SaveConfiguration (IO/SaveConfiguration.cpp:3-56): <OutputDirectory><Ufname>ID<seed>.txt and the E file
inline void SaveConfiguration(const std::string &Ufname, const std::string &Efname, GaugeLinks *U,
                              ElectricFields *E) {
    const std::string seed = std::to_string(RandomNumberGenerator::MySEED);
    const std::string uf = OutputDirectory + Ufname + "ID" + seed + ".txt";
    const std::string ef = OutputDirectory + Efname + "ID" + seed + ".txt";
    tcym_compat::check(tcym_lattice_save(tcym_compat::bind(U, E), uf.c_str(), ef.c_str()), "save configuration");
}
inline void SaveConfiguration(const std::string &Ufname, const std::string &Efname) {
    SaveConfiguration(Ufname, Efname, GLinks::U, EFields::E);
}
// LoadConfiguration (IO/LoadConfiguration.cpp:3-120): <InputDirectory><InputUFile>, <InputDirectory><InputEFile>
inline void LoadConfiguration(GaugeLinks *U, ElectricFields *E) {
    const std::string uf = InputDirectory + InputUFile, ef = InputDirectory + InputEFile;
    // after bind() the device copy is the newest; the host mirrors pull it on their next Get()
    tcym_compat::check(tcym_lattice_load(tcym_compat::bind(U, E), uf.c_str(), ef.c_str()), "load configuration");
}
inline void LoadConfiguration() { LoadConfiguration(GLinks::U, EFields::E); }
}  // namespace IO

namespace Observables {
namespace Bulk {
inline DOUBLE ESqr[3], BSqr[3];
inline void Update(GaugeLinks *U, ElectricFields *E) {
    tcym_obs o = tcym_compat::observables(U, E);
    for (int i = 0; i < 3; ++i) { ESqr[i] = o.esqr[i]; BSqr[i] = o.bsqr[i]; }
}
inline void Update() { Update(GLinks::U, EFields::E); }
// BulkObservables.cpp:29-51 with cE = cB = 1 (unit spacings, Minkowski metric)
inline DOUBLE T00() { return 0.5 * (ESqr[0] + ESqr[1] + ESqr[2] + BSqr[0] + BSqr[1] + BSqr[2]); }
inline DOUBLE TXX() { return 0.5 * ((ESqr[1] + ESqr[2] + BSqr[1] + BSqr[2]) - (ESqr[0] + BSqr[0])); }
inline DOUBLE TYY() { return 0.5 * ((ESqr[0] + ESqr[2] + BSqr[0] + BSqr[2]) - (ESqr[1] + BSqr[1])); }
inline DOUBLE TZZ() { return 0.5 * ((ESqr[0] + ESqr[1] + BSqr[0] + BSqr[1]) - (ESqr[2] + BSqr[2])); }
inline DOUBLE ELECTRIC() { return 0.5 * (ESqr[0] + ESqr[1] + ESqr[2]); }
inline DOUBLE MAGNETIC() { return 0.5 * (BSqr[0] + BSqr[1] + BSqr[2]); }
}  // namespace Bulk
namespace GaussLaw {
inline DOUBLE GlobalMaxViolation = 0.0, GlobalAvgViolation = 0.0;
inline void UpdateViolation(INT xl, INT xh, INT yl, INT yh, INT zl, INT zh, GaugeLinks *U, ElectricFields *E) {
    tcym_compat::whole(U, xl, xh, yl, yh, zl, zh);
    tcym_obs o = tcym_compat::observables(U, E);
    GlobalMaxViolation = o.gauss_max;
    GlobalAvgViolation = o.gauss_rms;
}
inline void CheckViolation(GaugeLinks *U, ElectricFields *E) {
    UpdateViolation(0, U->N[0] - 1, 0, U->N[1] - 1, 0, U->N[2] - 1, U, E);
    std::cerr << "#GAUSS LAW VIOLATION AT T=" << Dynamics::Time() << " MAX=" << GlobalMaxViolation
              << " AVG=" << GlobalAvgViolation << std::endl;
}
inline void CheckViolation() { CheckViolation(GLinks::U, EFields::E); }
}  // namespace GaussLaw
namespace Unitarity {
inline DOUBLE GlobalMaxViolation = 0.0, GlobalAvgViolation = 0.0;
inline void UpdateViolation(INT xl, INT xh, INT yl, INT yh, INT zl, INT zh, GaugeLinks *U) {
    tcym_compat::whole(U, xl, xh, yl, yh, zl, zh);
    tcym_obs o = tcym_compat::observables(U, U->binding ? U->binding->E : nullptr);
    GlobalMaxViolation = o.unit_max;
    GlobalAvgViolation = o.unit_rms;
}
inline void CheckViolation(GaugeLinks *U) {
    UpdateViolation(0, U->N[0] - 1, 0, U->N[1] - 1, 0, U->N[2] - 1, U);
    std::cerr << "#UNITARITY VIOLATION AT T=" << Dynamics::Time() << " MAX=" << GlobalMaxViolation
              << " AVG=" << GlobalAvgViolation << std::endl;
}
inline void CheckViolation() { CheckViolation(GLinks::U); }
}  // namespace Unitarity
}  // namespace Observables
