/*
 * A reference-style C++ caller of the drop-in classes: reads fsph_params
 * (raw struct bytes) and a particle file in the reference's binary format,
 * advances `steps` PBF steps through rxPBDSPH::Update, and writes the state
 * back with OutputParticles.  Used by tests/test_gpu_cpp_mirror.py.
 *
 *   pbf_driver params.bin in.dat out.dat steps dt
 */
#include <cstdio>
#include <cstdlib>

#include "fsph_particle_system.hpp"

int main(int argc, char **argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s params.bin in.dat out.dat steps dt\n", argv[0]);
        return 2;
    }
    fsph_params p;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f || std::fread(&p, sizeof(p), 1, f) != 1) { std::fprintf(stderr, "bad params\n"); return 2; }
    std::fclose(f);
    fsph_gb300::rxPBDSPH ps(p);
    if (!ps.IsInitialized()) { std::fprintf(stderr, "create: %s\n", ps.LastError().c_str()); return 1; }
    if (!ps.InputParticles(argv[2])) { std::fprintf(stderr, "input: %s\n", ps.LastError().c_str()); return 1; }
    const int steps = std::atoi(argv[4]);
    const float dt = (float)std::atof(argv[5]);
    for (int s = 0; s < steps; ++s) {
        if (!ps.Update(dt, s)) { std::fprintf(stderr, "update: %s\n", ps.LastError().c_str()); return 1; }
        std::printf("step %d iterations %d error %.6e\n", s, ps.GetIterations(), ps.GetDensityError());
    }
    ps.SetParticlesToCell();
    size_t total = 0;
    for (const auto &row : ps.GetNeights()) total += row.size();
    std::printf("neighbours %zu\n", total);
    if (!ps.OutputParticles(argv[3])) { std::fprintf(stderr, "output failed\n"); return 1; }
    return 0;
}
