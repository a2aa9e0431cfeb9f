// A dam break with a jet, written only against the reference's public API
// (FluidDomain, FluidSource, FluidSolverMemoryPool, FluidSolver,
// MarkerParticleSet), in the shape of the reference's substep loops
// (examples/simple.cpp, examples/opengl_example/FluidRendererGL.cpp:130-141).
// The same source compiles against the reference's own headers and against
// the GPU drop-in headers.
//
//   dam_break <steps> <particles.bin>
// writes the final particles as float32 {x, y, vx, vy} records.
#include <FluidDomain.h>
#include <FluidSolver.h>

#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

int main(int argc, char** argv)
{
    const int steps = argc > 1 ? std::atoi(argv[1]) : 50;
    const char* out = argc > 2 ? argv[2] : "particles.bin";
    const int n = 64;
    const MyFloat dt = 0.005;

    FluidDomain domain(n, n, n, n, 0.005, 0.02);
    FluidSolverMemoryPool pool(domain);
    FluidSolver solver(pool);
    // A block of fluid released at t = 0 and a jet spawning six times.
    domain.addFluidSource(FluidSource({2.0, 24.0, 2.0, 36.0}, 1.0, 1.0, 0.0, 0.0, 0.0, 1));
    domain.addFluidSource(FluidSource({2.0, 5.0, 48.0, 52.0}, 1.0, 1.0, 6.0, 0.0, 0.05, 6));
    try {
        for (int s = 0; s < steps; ++s) {
            domain.update(dt);
            solver.stepPICFLIP(domain, dt);
        }
    } catch (const std::runtime_error& e) {
        std::printf("error: %s\n", e.what());
        return 1;
    }
    const MarkerParticleSet& ps = domain.markerParticleSet();
    std::vector<float> buf;
    buf.reserve(4 * static_cast<size_t>(ps.size()));
    for (auto it = ps.begin(); it != ps.end(); ++it) {
        buf.push_back(it->posX());
        buf.push_back(it->posY());
        buf.push_back(it->velX());
        buf.push_back(it->velY());
    }
    std::FILE* f = std::fopen(out, "wb");
    if (!f) return 2;
    std::fwrite(buf.data(), sizeof(float), buf.size(), f);
    std::fclose(f);
    std::printf("%d particles after %d steps; cell (10, 5) is %d\n", ps.size(), steps,
                static_cast<int>(domain.macGrid().cellType(10, 5)));
    return 0;
}
