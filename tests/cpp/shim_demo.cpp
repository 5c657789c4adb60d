// A scene written the way Ziran's examples are (a falling corotated cube over a sticky ground,
// cf. Projects/anisofracture/examples/*.h), against the C++ shim ziran_gb300.hpp. Prints the particle
// count, the simulated time and the y-momentum after 20 substeps.
#include "ziran_gb300.hpp"

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
    return 0;
}
