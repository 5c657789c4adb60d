// A scene written the way Ziran's examples are (a falling corotated cube over a sticky ground,
// cf. Projects/anisofracture/examples/*.h), against the C++ shim ziran_gb300.hpp. Prints the particle
// count, the simulated time and the y-momentum after 20 substeps.
#include "ziran_gb300.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>

int main()
{
    using T = float;
    ziran_gb300::MpmSimulation<T> sim;
    sim.dx = (T)1 / 64;
    sim.dt = (T)1e-4;
    sim.gravity = { 0, (T)-9.8, 0 };
    sim.domain_cells = 68;
    std::vector<double> x, m, V0, v;
    std::mt19937 g(5);
    std::uniform_real_distribution<double> U(0, 1);
    const double dx = 1.0 / 64, vol = dx * dx * dx / 8;
    for (int i = 0; i < 8; i++)
        for (int j = 0; j < 8; j++)
            for (int k = 0; k < 8; k++)
                for (int s = 0; s < 8; s++) {
                    int sub[3] = { s >> 2, (s >> 1) & 1, s & 1 }, c[3] = { 28 + i, 34 + j, 28 + k };
                    for (int a = 0; a < 3; a++) x.push_back((c[a] + (sub[a] + U(g)) * 0.5) * dx);
                    m.push_back(1000 * vol);
                    V0.push_back(vol);
                    v.insert(v.end(), { 0.0, -1.0, 0.0 });
                }
    auto cube = sim.addParticles(x, m, V0, v);
    cube.addFBasedMpmForce(ziran_gb300::CorotatedElasticity<T>(1e4f, 0.3f));
    sim.addCollisionObject(ziran_gb300::HalfSpace<T>{ { 0, 0.05f, 0 }, { 0, 1, 0 } }, ziran_gb300::STICKY);
    sim.advance(20);
    std::vector<double> vel = sim.field(ZR_FIELD_V);
    double py = 0;
    for (size_t p = 0; p < m.size(); p++) py += m[p] * vel[3 * p + 1];
    std::printf("particles %lld time %.6f py %.9f\n", (long long)sim.particleCount(), sim.time(), py);

    // An AnisoMPM piece the way examples/tubepull.h builds one: QRStableNeoHookean with fibre stiffness
    // 10 mu along the material x axis and anisotropic damage, pulled apart by two sticky plates.
    // run twice: the explicit damage update, then AnisoFractureSimulation's implicit solve (sim.implicit)
    for (int implicit = 0; implicit < 2; implicit++) {
        ziran_gb300::MpmSimulation<T> tear;
        tear.implicit = implicit != 0;
        tear.dx = (T)1 / 128;
        tear.dt = (T)5e-5;
        tear.apic_rpic_ratio = 0;
        tear.domain_cells = 132;
        std::vector<double> xs, ms, vs, Fs;
        const double h = 1.0 / 128, vh = h * h * h / 8;
        for (int i = 0; i < 12; i++)
            for (int j = 0; j < 4; j++)
                for (int k = 0; k < 4; k++)
                    for (int s = 0; s < 8; s++) {
                        int sub[3] = { s >> 2, (s >> 1) & 1, s & 1 }, c[3] = { 58 + i, 62 + j, 62 + k };
                        for (int a = 0; a < 3; a++) xs.push_back((c[a] + (sub[a] + U(g)) * 0.5) * h);
                        ms.push_back(800 * vh);
                    }
        const size_t n2 = ms.size();
        std::vector<double> V2(n2, vh);
        ziran_gb300::QRStableNeoHookean<T> model(5e4f, 0.25f);
        model.setExtraFiberStiffness(0, 10);
        auto piece = tear.addParticles(xs, ms, V2);
        piece.addFBasedMpmForce(model);
        std::vector<T> sc(n2, model.getSigmaCrit((T)0.01));
        piece.addFBasedMpmForceWithAnisotropicPhaseField((T)-1, (T)(0.5 * h), model, (T)0.1, (T)1, (T)0.01, sc);
        tear.addCollisionObject(ziran_gb300::HalfSpace<T>{ { (T)(60 * h), 0, 0 }, { 1, 0, 0 } }, ziran_gb300::STICKY, 0, { (T)-1, 0, 0 });
        tear.addCollisionObject(ziran_gb300::HalfSpace<T>{ { (T)(68 * h), 0, 0 }, { -1, 0, 0 } }, ziran_gb300::STICKY, 0, { (T)1, 0, 0 });
        tear.advance(30);
        std::vector<double> dmg = tear.field(ZR_FIELD_D);
        double dmax = 0;
        for (double v : dmg) dmax = v > dmax ? v : dmax;
        std::printf("qr_particles %lld max_damage %.6f cg %d\n", (long long)tear.particleCount(), dmax, tear.cgIterations());
    }

    // The cube's state as the input of two independent one-substep jobs (stepJobs pipelines them with their host
    // copies): both results are the same substep of the same state, up to the order of the atomic grid sums
    const size_t ns = (size_t)sim.particleCount() * 25;
    std::vector<T> st(ns), r0(ns), r1(ns);
    sim.getState(st.data());
    sim.stepJobs({ st.data(), st.data() }, { r0.data(), r1.data() });
    double jd = 0, moved = 0;
    for (size_t q = 0; q < ns; q += 25)
        for (int a = 0; a < 3; a++) {
            jd = std::max(jd, std::abs((double)r0[q + a] - (double)r1[q + a]));
            moved = std::max(moved, std::abs((double)r0[q + a] - (double)st[q + a]));
        }
    std::printf("jobs_diff %.3e moved %.3e reruns %lld\n", jd, moved, sim.stepJobsRerun());
    return 0;
}
