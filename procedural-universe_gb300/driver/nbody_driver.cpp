// nbody_driver.cpp -- headless precompute driver.
//
// The batch caller of the N-body step, as the reference's precompute mode
// (src/App/NBody.cpp:52-88, src/States/Simulation/SimulationState.cpp:279-332):
//
//   nbody_driver -c [-t simtime_s] [-s timestep] [-p particles] [-f file]
//
// seeds a star system (StarSystemSeeder) -- or loads data/<file>, re-centred
// on its centre of mass -- then steps the Barnes-Hut simulator with
// dt = timestep / 60 until simtime seconds of wall clock have passed, logging
// once a second, and writes the particles to data/<ticks>.nbody.  Physics
// constants are the reference's (G = 6.674e-11, S = 10, drift divided by
// StarSystemScale = 2.3e13, theta = 2.0) unless --nbody-units selects
// G = 1, eps = 0.01, no drift scale, theta = 0.5.  --steps k runs exactly k
// steps instead of the wall-clock budget (for reproducible runs).
//
// Deviation: the reference seeds after loading a file, which overwrites the
// loaded particles; here a loaded file is simulated as loaded.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "cuda_nbody_sim.hpp"

namespace {

void usage() {
    std::fprintf(stderr,
                 "usage: nbody_driver -c [-t simtime_s] [-s timestep] [-p particles] [-f file]\n"
                 "                       [--steps k] [--direct] [--nbody-units] [--out path] [--device d] [--seed s]\n");
}

}  // namespace

int main(int argc, char** argv) {
    bool compute = false, nbody_units = false, direct = false;
    int simtime = 10, particles = 4000, device = 0;
    long max_steps = -1;   // --steps k: exactly k steps instead of a wall-clock budget
    float timestep = 0.02f;
    unsigned long long seed = 0;
    std::string file, out;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&](const char* name) -> const char* {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "missing value for %s\n", name);
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "-c" || a == "--compute") compute = true;
        else if (a == "-t" || a == "--simtime") simtime = std::atoi(next("-t"));
        else if (a == "-s" || a == "--timestep") timestep = (float)std::atof(next("-s"));
        else if (a == "-p" || a == "--particles") particles = std::atoi(next("-p"));
        else if (a == "-f" || a == "--file") file = next("-f");
        else if (a == "--out") out = next("--out");
        else if (a == "--device") device = std::atoi(next("--device"));
        else if (a == "--seed") seed = std::strtoull(next("--seed"), nullptr, 10);
        else if (a == "--steps") max_steps = std::atol(next("--steps"));
        else if (a == "--nbody-units") nbody_units = true;
        else if (a == "--direct") direct = true;
        else {
            usage();
            return 2;
        }
    }
    if (!compute) {
        usage();
        return 2;
    }
    if (particles < 1 || simtime < 0) {
        std::fprintf(stderr, "bad -p or -t\n");
        return 2;
    }
    std::vector<nb_particle> p;
    if (!file.empty()) {
        const std::string path = "data/" + file;
        size_t n = 0;
        if (nb_file_read(path.c_str(), nullptr, 0, &n, 0) != NB_OK || n == 0) {
            std::fprintf(stderr, "Could not read particle file %s\n", file.c_str());
            return 1;
        }
        p.resize(n);
        if (nb_file_read(path.c_str(), p.data(), n, &n, 1) != NB_OK) {
            std::fprintf(stderr, "Could not read particle file %s\n", file.c_str());
            return 1;
        }
        std::printf("Read %zu particles from file\n", n);
    } else {
        p.resize((size_t)particles);
        nb_seed_reference(2, seed, 1.0f, p.data(), p.size());
    }
    nb_params prm;
    nb_default_params(&prm);
    prm.device = device;
    if (nbody_units) {
        prm.G = 1.0;
        prm.softening2 = 1e-4;
        prm.pos_scale = 1.0;
        prm.theta = 0.5;
    } else {
        prm.G = 6.674e-11;     // Phys::G
        prm.softening2 = 10.0; // Phys::S
        prm.pos_scale = 20 * 1.15e12;   // Phys::StarSystemScale
        prm.theta = 2.0;       // Octree::Theta before any UI change
    }
    const float dt = timestep * (1.0f / 60.0f);
    long iterations = 0;
    try {
        auto sim = nbgb::CreateNBodySim(direct ? nbgb::ENBodySim::BruteForceCPU : nbgb::ENBodySim::BarnesHut, &prm);
        sim->Init(p);
        const auto start = std::chrono::steady_clock::now();
        auto tick = start;
        while (true) {
            ++iterations;
            const auto now = std::chrono::steady_clock::now();
            if (max_steps >= 0 ? iterations > max_steps
                               : std::chrono::duration<double>(now - start).count() >= simtime)
                break;
            if (std::chrono::duration<double>(now - tick).count() >= 1.0) {
                tick = now;
                std::printf("Running... (%ld iterations)\n", iterations);
                std::fflush(stdout);
            }
            sim->Update(dt);
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
        if (out.empty()) {
            mkdir("data", 0755);
            const long long ticks = (long long)std::chrono::steady_clock::now().time_since_epoch().count();
            out = "data/" + std::to_string(ticks) + ".nbody";
        }
        if (nb_file_write(out.c_str(), p.data(), p.size()) != NB_OK) {
            std::fprintf(stderr, "could not write %s\n", out.c_str());
            return 1;
        }
        std::printf("{\"file\": \"%s\", \"bodies\": %zu, \"steps\": %ld, \"seconds\": %.3f, \"body_steps_per_s\": %.6e}\n",
                    out.c_str(), p.size(), iterations - 1, secs, (double)p.size() * (iterations - 1) / (secs > 0 ? secs : 1));
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
