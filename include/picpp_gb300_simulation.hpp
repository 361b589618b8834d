// picpp_gb300_simulation.hpp -- header-only C++ mirror of the hot-path member
// functions of PIC++'s class Simulation (PIC++/simulation.h:32-1152) over the
// C ABI of picpp_gb300.h.  A C++ caller that used Simulation's step loop
// (PIC++/simulation.cpp:164-259) keeps the same call sequence:
//
//   picpp::GpuSimulation sim(cfg);
//   sim.addSpecies(q, m, w, n); sim.uploadParticles(0, ...); sim.uploadFields(E, B);
//   sim.tristanEvaluateBhalfStep(); sim.moveParticles(); sim.tristanEvaluateBhalfStep();
//   sim.tristanUpdateFlux(); sim.tristanEvaluateE();
//
// Errors throw picpp::Error (status + message) instead of the reference's
// print-and-exit (PIC++/util.cpp:119-129).
#pragma once
#include <stdexcept>
#include <string>
#include <vector>

#include "picpp_gb300.h"

namespace picpp {

class Error : public std::runtime_error {
public:
    Error(pic_status s, const std::string& m) : std::runtime_error(m), status(s) {}
    pic_status status;
};

class GpuSimulation {
public:
    explicit GpuSimulation(const pic_config& cfg) {
        pic_status s = pic_create(&cfg, &ctx_);
        if (s != PIC_OK) throw Error(s, "pic_create failed");
    }
    ~GpuSimulation() { pic_destroy(ctx_); }
    GpuSimulation(const GpuSimulation&) = delete;
    GpuSimulation& operator=(const GpuSimulation&) = delete;

    pic_ctx* handle() const { return ctx_; }

    int addSpecies(double q, double m, double w, long capacity) {
        int id = -1;
        check(pic_add_species(ctx_, q, m, w, capacity, &id));
        return id;
    }
    void uploadParticles(int species, long n, const int* cell, const double* ox, const double* oy, const double* oz,
                         const double* px, const double* py, const double* pz, const int* ids = nullptr) {
        check(pic_upload_particles(ctx_, species, n, cell, ox, oy, oz, px, py, pz, ids));
    }
    long downloadParticles(int species, int* cell, double* ox, double* oy, double* oz, double* px, double* py,
                           double* pz, int* ids = nullptr) {
        long n = 0;
        check(pic_download_particles(ctx_, species, &n, cell, ox, oy, oz, px, py, pz, ids));
        return n;
    }
    // injectNewParticles (PIC++/mover.cpp:910-1000) with the caller's new
    // particles, appended after the species' own
    void injectNewParticles(int species, long n, const int* cell, const double* ox, const double* oy,
                            const double* oz, const double* px, const double* py, const double* pz,
                            const int* ids = nullptr) {
        check(pic_append_particles(ctx_, species, n, cell, ox, oy, oz, px, py, pz, ids));
    }
    // device loading of a drifting Maxwell-Juttner species (no reference counterpart)
    void fillSpecies(int species, int ppc, unsigned long long seed, double theta, double drift_gamma,
                     int alternate_drift) {
        check(pic_fill_species(ctx_, species, ppc, seed, theta, drift_gamma, alternate_drift));
    }
    void uploadFields(const double* E, const double* B) { check(pic_upload_fields(ctx_, E, B)); }
    void downloadFields(double* E, double* B, double* J) { check(pic_download_fields(ctx_, E, B, J)); }

    // explicit Buneman / Tristan phases (PIC++/simulation.cpp:164-204)
    void tristanEvaluateBhalfStep() { check(pic_tristan_evaluate_b_half_step(ctx_)); }
    void moveParticles() { check(pic_move_particles(ctx_)); }
    void tristanUpdateFlux() { check(pic_tristan_update_flux(ctx_)); }
    void tristanEvaluateE() { check(pic_tristan_evaluate_e(ctx_)); }
    void bunemanSteps(int n) { check(pic_buneman_step(ctx_, n)); }

    // implicit phases (PIC++/simulation.cpp:205-259).  The rotation tensor
    // of evaluateParticlesRotationTensor is recomputed inside the deposit and
    // the mover, so that call has nothing left to do on its own.
    void evaluateParticlesRotationTensor() {}
    void updateElectroMagneticParameters() { check(pic_update_electromagnetic_parameters(ctx_)); }
    pic_solve_info evaluateElectricField(const pic_solve_opts& opts = defaultSolve()) {
        pic_solve_info info{};
        pic_status s = pic_evaluate_electric_field(ctx_, &opts, &info);
        if (s != PIC_OK && s != PIC_ERR_NOT_CONVERGED) check(s);
        return info;
    }
    void evaluateMagneticField() { check(pic_evaluate_magnetic_field(ctx_)); }
    void updateFields() { check(pic_update_fields(ctx_)); }
    // the whole implicit branch of one step
    pic_solve_info implicitStep(const pic_solve_opts& opts = defaultSolve()) {
        pic_solve_info info{};
        pic_status s = pic_implicit_step(ctx_, &opts, &info);
        if (s != PIC_OK && s != PIC_ERR_NOT_CONVERGED) check(s);
        return info;
    }
    // escaped particles of a wall box are erased inside the step calls
    // (the next sort, before any call that reads particles)
    void eraseEscapedPaticles() {}
    // correlation maps and the periodic particle exchange are folded into
    // the kernels (cell index + offset, wrap on every move)
    void updateParticleCorrelationMaps() {}
    void exchangeParticles() {}
    void sortParticles() { check(pic_sort_particles(ctx_)); }

    // outputBackup / readBackup (PIC++/simulation.cpp:921-933, input.cpp:342-624)
    void outputBackup(const std::string& path) { check(pic_save_checkpoint(ctx_, path.c_str())); }
    void readBackup(const std::string& path) { check(pic_load_checkpoint(ctx_, path.c_str())); }

    // updateDensityParameters (PIC++/momentum_collecting.cpp:760-1020)
    void updateDensityParameters() { check(pic_update_density_parameters(ctx_)); }

    // updateEnergy (PIC++/simulation.cpp:1506-1600)
    std::vector<double> updateEnergy() {
        std::vector<double> out(6);
        check(pic_energy(ctx_, out.data()));
        return out;
    }

    // learned right preconditioner of PIC_FGMRES_LEARNED (no reference
    // counterpart): initialise or load, train on the current operator
    void initPreconditioner(unsigned long long seed) { check(pic_nn_init(ctx_, seed)); }
    void loadPreconditioner(const std::vector<float>& p) {
        if ((long)p.size() != pic_nn_param_count()) throw Error(PIC_ERR_ARG, "wrong parameter count");
        check(pic_nn_set_params(ctx_, p.data()));
    }
    std::vector<float> savePreconditioner() {
        std::vector<float> p((size_t)pic_nn_param_count());
        check(pic_nn_get_params(ctx_, p.data()));
        return p;
    }
    pic_train_info trainPreconditioner(const pic_train_opts& opts) {
        pic_train_info info{};
        check(pic_nn_train(ctx_, &opts, &info));
        return info;
    }
    // record up to capacity (right part, mu, solution) triples of the plain
    // solves that follow (pic_train_opts.source = 1 trains on them)
    void recordSolves(int capacity) { check(pic_nn_record(ctx_, capacity)); }
    int recordedSolves() {
        int n = 0;
        check(pic_nn_record_count(ctx_, &n));
        return n;
    }
    // bound of the convolutions' MMA-completion waits (0: the built-in one)
    void convolutionWaitLimit(unsigned polls) { check(pic_nn_wait_limit(ctx_, polls)); }

    // per-phase device time (the reference's timing prints)
    void profile(bool enable, double* phase_ms = nullptr, long* launches = nullptr) {
        check(pic_profile(ctx_, enable ? 1 : 0, phase_ms, launches));
    }

    static pic_solve_opts defaultSolve() { return pic_solve_opts{PIC_GMRES_REFERENCE, 30, 50, 1e-8}; }

private:
    void check(pic_status s) {
        if (s != PIC_OK) throw Error(s, pic_last_error(ctx_));
    }
    pic_ctx* ctx_ = nullptr;
};

}  // namespace picpp
