// GpuFlameSolver: Ember's FlameSolver with its two stage hooks on the GB300
// library (include/ember_gpu.h). Selected by General.chemistryIntegrator =
// "gpu-qss" or "gpu-bdf" (ember-gpu.patch makes the Python layer construct it).
//
//   integrateProductionTerms  FlameSolver::integrateProductionTerms
//                             (src/flameSolver.cpp:754-836): every grid point's
//                             source system in one ember_source_integrate call;
//   integrateDiffusionTerms   FlameSolver::integrateDiffusionTerms
//                             (src/flameSolver.cpp:838-854): every state
//                             variable's DiffusionSystem in one
//                             ember_diffusion_integrate call, with the step-size
//                             rule of setDiffusionSolverState (702-718).
//
// Everything else (properties, convection, grid, output) is FlameSolver's.
// The mechanism is compiled once from the Cantera objects of the run's
// mechanism file (ember_mech_create): NASA7 thermo of every species and, per
// reaction, its Arrhenius (or falloff) parameters, third-body efficiencies and
// species occurrences. Written against Ember's headers and Cantera 3.x; it is
// not compiled in this repository (Ember, Cantera, Eigen and Boost are not
// available where the library is built).
#pragma once

#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "cantera/base/Solution.h"
#include "cantera/kinetics/Falloff.h"
#include "cantera/kinetics/Kinetics.h"
#include "cantera/kinetics/Reaction.h"
#include "cantera/thermo/NasaPoly2.h"
#include "cantera/thermo/ThermoPhase.h"
#include "ember_gpu.h"
#include "flameSolver.h"

class GpuFlameSolver : public FlameSolver
{
public:
    ~GpuFlameSolver() override {
        if (mech_) ember_mech_destroy(mech_);
    }

    // FlameSolver::setOptions is not virtual: the GPU settings are read from
    // the stored options on first use.
    void configure() {
        const ConfigOptions& o = options;
        method_ = (o.chemistryIntegrator == "gpu-bdf") ? EMBER_SOURCE_BDF : EMBER_SOURCE_QSS;
        ember_source_options_default(&src_);
        src_.pressure = o.pressure;
        src_.kinetics_model = (o.kineticsModel == "standard") ? EMBER_KINETICS_STANDARD : EMBER_KINETICS_INTERP;
        src_.qss_epsmin = o.qss_epsmin;
        src_.qss_epsmax = o.qss_epsmax;
        src_.qss_dtmin = o.qss_dtmin;
        src_.qss_dtmax = o.qss_dtmax;
        src_.qss_abstol = o.qss_abstol;
        src_.qss_minval = o.qss_minval;
        src_.qss_iteration_count = o.qss_iterationCount;
        src_.qss_stability_check = o.qss_stabilityCheck;
        src_.bdf_reltol = o.integratorRelTol;
        src_.bdf_abstol_momentum = o.integratorMomentumAbsTol;
        src_.bdf_abstol_energy = o.integratorEnergyAbsTol;
        src_.bdf_abstol_species = o.integratorSpeciesAbsTol;
        src_.bdf_min_step = o.integratorMinTimestep;
    }

    void integrateProductionTerms() override {
        ensureMechanism();
        std::vector<double> dt(nPoints, tStageEnd - tStageStart);
        std::vector<int> status(nPoints);
        // state and splitConstProd are nVars x nPoints column-major: the [points][nVars] layout of the ABI
        const int rc = ember_source_integrate(mech_, method_, int(nPoints), state.data(), splitConstProd.data(),
                                              dt.data(), tStageStart, x.data(), &src_, state.data(), status.data(),
                                              nullptr, EMBER_MEM_HOST, nullptr);
        if (rc != EMBER_OK && rc != EMBER_EFAIL) throw std::runtime_error(lastError("ember_source_integrate"));
        for (size_t j = 0; j < nPoints; j++) {
            if (status[j] != 0) {
                logFile.write(format("GPU source term: integration failed at j = %i (status %i)") % j % status[j]);
            }
        }
    }

    void integrateDiffusionTerms() override {
        // rows of every variable: B, D, split constant (prepareIntegrators) and the state row
        const size_t N = nPoints;
        B_.resize(nVars * N);
        D_.resize(nVars * N);
        S_.resize(nVars * N);
        Y_.resize(nVars * N);
        wall_.assign(nVars, 0.0);
        yinf_.assign(nVars, 0.0);
        for (size_t k = 0; k < nVars; k++) {
            for (size_t j = 0; j < N; j++) {
                B_[k * N + j] = diffusionTerms[k].B[j];
                D_[k * N + j] = diffusionTerms[k].D[j];
                S_[k * N + j] = diffusionTerms[k].splitConst[j];
                Y_[k * N + j] = state(k, j);
            }
            wall_[k] = diffusionTerms[k].wallConst;
            yinf_[k] = diffusionTerms[k].yInf;
        }
        ember_diffusion_grid g = {int(N), int(grid.leftBC), int(grid.rightBC), grid.alpha};
        ember_diffusion_options o = {tStageStart, tStageEnd, options.diffusionTimestepMultiplier,
                                     options.globalTimestep, nullptr, wall_.data(), yinf_.data(),
                                     EMBER_DIFFUSION_PARALLEL};
        status_.resize(nVars);
        const int rc = ember_diffusion_integrate(1, &g, int(nVars), x.data(), B_.data(), D_.data(), S_.data(),
                                                 Y_.data(), &o, status_.data(), EMBER_MEM_HOST, nullptr);
        if (rc != EMBER_OK && rc != EMBER_EFAIL) throw std::runtime_error(lastError("ember_diffusion_integrate"));
        for (size_t k = 0; k < nVars; k++) {
            for (size_t j = 0; j < N; j++) {
                state(k, j) = Y_[k * N + j];
            }
        }
    }

private:
    static std::string lastError(const char* what) {
        char buf[1024];
        ember_last_error(buf, sizeof buf);
        return std::string(what) + ": " + buf;
    }

    // Species occurrences of one side of a reaction, each stoichiometric unit once (up to EMBER_MAX_STOICH).
    static void occurrences(const Cantera::Composition& side, const Cantera::ThermoPhase& th, int* out) {
        int n = 0;
        for (int o = 0; o < EMBER_MAX_STOICH; o++) out[o] = -1;
        for (const auto& sp : side) {
            const double nu = sp.second;
            if (nu != std::round(nu)) throw std::runtime_error("non-integer stoichiometry: " + sp.first);
            for (int u = 0; u < int(nu); u++) {
                if (n == EMBER_MAX_STOICH) throw std::runtime_error("more than 4 species occurrences on one side");
                out[n++] = int(th.speciesIndex(sp.first));
            }
        }
    }

    // Arrhenius parameters in Cantera's internal units, activation energy as Ea / R.
    static void arrhenius(const Cantera::ArrheniusRate& r, double* p) {
        p[0] = r.preExponentialFactor();
        p[1] = r.temperatureExponent();
        p[2] = r.activationEnergy() / Cantera::GasConstant;
    }

    void ensureMechanism() {
        if (mech_) return;
        configure();
        auto sol = Cantera::newSolution(options.gasMechanismFile, options.gasPhaseID, "none");
        auto th = sol->thermo();
        auto kin = sol->kinetics();
        const int S = int(th->nSpecies()), R = int(kin->nReactions());
        std::vector<double> W(S), tmid(S), nasa(14 * size_t(S));
        for (int k = 0; k < S; k++) {
            W[k] = th->molecularWeight(k);
            size_t n;
            int type;
            double tlow, thigh, pref, c[15];
            th->species(k)->thermo->reportParameters(n, type, tlow, thigh, pref, c);
            tmid[k] = c[0];                                  // NasaPoly2: [Tmid, high a0..a6, low a0..a6]
            for (int i = 0; i < 7; i++) {
                nasa[14 * k + i] = c[8 + i];                 // low range first in ember_mech_desc
                nasa[14 * k + 7 + i] = c[1 + i];
            }
        }
        std::vector<int> type(R), rev(R), reac(4 * size_t(R)), prod(4 * size_t(R));
        std::vector<double> arr(3 * size_t(R), 0.0), low(3 * size_t(R), 0.0), troe(4 * size_t(R), 0.0), def(R, 1.0);
        std::vector<int64_t> eoff(R + 1, 0);
        std::vector<int> esp;
        std::vector<double> eval;
        for (int i = 0; i < R; i++) {
            auto rx = kin->reaction(i);
            rev[i] = rx->reversible ? 1 : 0;
            occurrences(rx->reactants, *th, &reac[4 * i]);
            occurrences(rx->products, *th, &prod[4 * i]);
            auto rate = rx->rate();
            if (auto fo = std::dynamic_pointer_cast<Cantera::FalloffRate>(rate)) {
                arrhenius(fo->highRate(), &arr[3 * i]);
                arrhenius(fo->lowRate(), &low[3 * i]);
                std::vector<double> c;
                fo->getFalloffCoeffs(c);
                type[i] = c.empty() ? EMBER_RXN_LINDEMANN : EMBER_RXN_TROE;
                for (size_t q = 0; q < c.size() && q < 4; q++) troe[4 * i + q] = c[q];
            } else if (auto ar = std::dynamic_pointer_cast<Cantera::ArrheniusRate>(rate)) {
                arrhenius(*ar, &arr[3 * i]);
                type[i] = rx->usesThirdBody() ? EMBER_RXN_THREE_BODY : EMBER_RXN_ELEMENTARY;
            } else {
                throw std::runtime_error("reaction " + rx->equation() + ": rate type not supported on the GPU");
            }
            if (rx->usesThirdBody()) {
                auto tb = rx->thirdBody();
                def[i] = tb->default_efficiency;
                for (const auto& e : tb->efficiencies) {
                    esp.push_back(int(th->speciesIndex(e.first)));
                    eval.push_back(e.second);
                }
            }
            eoff[i + 1] = int64_t(esp.size());
        }
        ember_mech_desc d = {S, R, W.data(), tmid.data(), nasa.data(), type.data(), rev.data(), reac.data(),
                             prod.data(), arr.data(), low.data(), troe.data(), def.data(), eoff.data(),
                             esp.data(), eval.data()};
        if (ember_mech_create(&d, &mech_) != EMBER_OK) throw std::runtime_error(lastError("ember_mech_create"));
    }

    ember_mech mech_ = nullptr;
    int method_ = EMBER_SOURCE_QSS;
    ember_source_options src_{};
    std::vector<double> B_, D_, S_, Y_, wall_, yinf_;
    std::vector<int> status_;
};
