// mirror_steps.cpp -- a C++ caller of the drop-in: loads a state, runs the
// step loop through the Simulation-shaped C++ mirror (the member-function
// sequence of PIC++/simulation.cpp:164-259) and writes the result.  Built
// and run by tests/test_gpu_cpp_mirror.py, which checks the output against
// the oracle.
//
// Input (little endian): int32 nx ny nz solver particle_real steps nspecies
// pressure_compat; float64 dx dy dz dt theta eta cfix; per species float64
// q m w, int64 n, int32 cell[n], float64 ox oy oz px py pz [n] each, int32
// id[n]; float64 E[3N], B[3N].  Output: float64 E[3N], B[3N], then per
// species int64 n, int32 cell[n], float64 ox oy oz px py pz [n], int32 id[n].
#include <cstdint>
#include <cstdio>
#include <vector>

#include "picpp_gb300_simulation.hpp"

namespace {

template <typename T>
void rd(std::FILE* f, T* p, size_t n) {
    if (std::fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short input");
}
template <typename T>
void wr(std::FILE* f, const T* p, size_t n) {
    if (std::fwrite(p, sizeof(T), n, f) != n) throw std::runtime_error("short output");
}

struct Species {
    double q, m, w;
    int64_t n;
    std::vector<int> cell, id;
    std::vector<double> a[6];
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: mirror_steps in.bin out.bin\n");
        return 2;
    }
    try {
        std::FILE* in = std::fopen(argv[1], "rb");
        if (!in) throw std::runtime_error("cannot open input");
        int32_t h[8];
        double d[7];
        rd(in, h, 8);
        rd(in, d, 7);
        pic_config cfg{};
        cfg.nx = h[0]; cfg.ny = h[1]; cfg.nz = h[2];
        cfg.solver = h[3];
        cfg.particle_real = h[4];
        cfg.field_real = h[4];
        cfg.pressure_compat = h[7];
        cfg.sort_every = 1;
        cfg.dx = d[0]; cfg.dy = d[1]; cfg.dz = d[2]; cfg.dt = d[3];
        cfg.theta = d[4]; cfg.eta = d[5]; cfg.cfix = d[6];
        const int steps = h[5], ns = h[6];
        const size_t L = 3 * (size_t)cfg.nx * cfg.ny * cfg.nz;
        std::vector<Species> sp(ns);
        for (auto& s : sp) {
            rd(in, &s.q, 1); rd(in, &s.m, 1); rd(in, &s.w, 1);
            rd(in, &s.n, 1);
            s.cell.resize(s.n); s.id.resize(s.n);
            rd(in, s.cell.data(), s.n);
            for (auto& a : s.a) { a.resize(s.n); rd(in, a.data(), s.n); }
            rd(in, s.id.data(), s.n);
        }
        std::vector<double> E(L), B(L), J(L);
        rd(in, E.data(), L);
        rd(in, B.data(), L);
        std::fclose(in);

        picpp::GpuSimulation sim(cfg);
        for (int k = 0; k < ns; ++k) {
            Species& s = sp[k];
            const int id = sim.addSpecies(s.q, s.m, s.w, (long)s.n);
            sim.uploadParticles(id, (long)s.n, s.cell.data(), s.a[0].data(), s.a[1].data(), s.a[2].data(),
                                s.a[3].data(), s.a[4].data(), s.a[5].data(), s.id.data());
        }
        sim.uploadFields(E.data(), B.data());
        for (int it = 0; it < steps; ++it) {
            if (cfg.solver == PIC_SOLVER_BUNEMAN) {
                sim.tristanEvaluateBhalfStep();
                sim.moveParticles();
                sim.tristanEvaluateBhalfStep();
                sim.tristanUpdateFlux();
                sim.tristanEvaluateE();
            } else {
                sim.evaluateParticlesRotationTensor();
                sim.updateElectroMagneticParameters();
                pic_solve_opts o{PIC_GMRES_REFERENCE, 30, 50, 1e-8};
                sim.evaluateElectricField(o);
                sim.evaluateMagneticField();
                sim.moveParticles();
                sim.updateParticleCorrelationMaps();
                sim.updateFields();
            }
        }
        sim.downloadFields(E.data(), B.data(), J.data());
        std::FILE* out = std::fopen(argv[2], "wb");
        if (!out) throw std::runtime_error("cannot open output");
        wr(out, E.data(), L);
        wr(out, B.data(), L);
        for (int k = 0; k < ns; ++k) {
            Species& s = sp[k];
            const long n = sim.downloadParticles(k, s.cell.data(), s.a[0].data(), s.a[1].data(), s.a[2].data(),
                                                 s.a[3].data(), s.a[4].data(), s.a[5].data(), s.id.data());
            const int64_t n64 = n;
            wr(out, &n64, 1);
            wr(out, s.cell.data(), n);
            for (auto& a : s.a) wr(out, a.data(), n);
            wr(out, s.id.data(), n);
        }
        std::fclose(out);
    } catch (const picpp::Error& e) {
        std::fprintf(stderr, "picpp error %d: %s\n", (int)e.status, e.what());
        return 1;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
