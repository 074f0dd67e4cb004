// A driver written against the reference's C++ hot-path API (the shape of
// SphaleronSimulation.cpp's Init/Evolve), built on include/tcym_compat.hpp.
// Prints "key value..." lines that tests/test_gpu_compat.py compares with the oracle.
#include <cstdio>
#include <cstdlib>

#include "tcym_compat.hpp"

int main(int argc, char **argv) {
    const int L = argc > 1 ? std::atoi(argv[1]) : 8;
    Lattice::N[0] = Lattice::N[1] = Lattice::N[2] = L;
    Lattice::Volume = L * L * L;
    Lattice::Init();
    InitialConditions::SetZero();
    RandomNumberGenerator::MySEED = 1;
    ThermalDynamics::beta = 2.0;
    ThermalDynamics::ReassignElectricFields();
    Observables::GaussLaw::CheckViolation();
    Dynamics::dTau = 0.05;
    for (int rec = 0; rec <= 5; ++rec) {
        Observables::Bulk::Update();
        std::printf("bulk %d %.17g %.17g %.17g\n", Dynamics::tSteps, Observables::Bulk::T00(),
                    Observables::Bulk::ELECTRIC(), Observables::Bulk::MAGNETIC());
        if (rec < 5)
            for (int s = 0; s < 10; ++s) Dynamics::Update();
    }
    // host access to the state through the reference's accessors
    std::printf("link %.17g\n", (double)std::real(*GLinks::U->Get(1, 2, 3, 1)));
    std::printf("field %.17g\n", *EFields::E->Get(2, 1, 0, 2, 1));
    std::printf("edotb %.17g %.17g\n", UnimprovedOperators::ComputeEDotB(GLinks::U, EFields::E),
                ImprovedOperators::ComputeEDotB(GLinks::U, EFields::E));
    Observables::Unitarity::CheckViolation();
    std::printf("unitarity %.17g\n", Observables::Unitarity::GlobalMaxViolation);
    // Langevin steps (beta = 1/T)
    LangevinDynamics::beta = 1.0 / 0.6;
    LangevinDynamics::dTauL = 0.02;
    RandomNumberGenerator::MySEED = 3;
    for (int s = 0; s < 5; ++s) LangevinDynamics::Update();
    Observables::Bulk::Update();
    std::printf("langevin %.17g\n", Observables::Bulk::T00());
    // cooling: flow a copy, then calibrated flow on the fields
    GaugeLinks UCold(L, L, L, 1, 1, 1);
    GradientFlow::SqrtDcTauOverSpacing = 0.1414213562373095;  // dtau = 0.02
    Cooling::CoolNSave("cool", 5, 0, GLinks::U, &UCold);
    std::printf("cooled %.17g\n", (double)std::real(*UCold.Get(0, 0, 0, 0)));
    ChernSimonsNumber::DeltaNCsCooling = 0.0;
    GradientFlow::Reset();
    for (int s = 0; s < 3; ++s) GradientFlow::CalibrationUpdate(GLinks::U, EFields::E);
    std::printf("calibration %.17g %.17g\n", ChernSimonsNumber::DeltaNCsCooling, GradientFlow::CoolingTime());
    // blocked cooling: one Block (after 2 of 6 steps) onto L/2 extents, spacing 2
    Cooling::BlockFrequency = 2;
    GaugeLinks UBlocked(L / 2, L / 2, L / 2, 2, 2, 2);
    Cooling::CoolNSave("coolb", 6, 1, GLinks::U, &UBlocked);
    std::printf("cooled_blocked %.17g %.17g\n", (double)std::real(*UBlocked.Get(0, 0, 0, 0)),
                (double)std::real(*UBlocked.Get(1, 2, 2, 2)));
    // cooled real-time N_CS at StandardBlockingLevel 1
    ChernSimonsNumber::CoolingMethod::StandardBlockingLevel = 1;
    ChernSimonsNumber::CoolingMethod::StandardCoolingMaxSteps = 6;
    ChernSimonsNumber::CoolingMethod::Init();
    ChernSimonsNumber::CoolingMethod::Start();
    for (int s = 0; s < 10; ++s) Dynamics::Update();
    ChernSimonsNumber::CoolingMethod::Update(1);
    std::printf("cooled_ncs %.17g\n", ChernSimonsNumber::DeltaNCsCoolRealTime);
    return 0;
}
