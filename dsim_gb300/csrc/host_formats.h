// host_formats.h -- the reference's input formats, parsed on the host.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>

namespace dsim {

// Mesh fiber file after SpinSystem::initFibers (dSim3/src/spinSystem.cpp:290-673)
struct MeshHost {
    std::vector<float> vertices;     // 3V, divided by spaceScale
    std::vector<uint32_t> trgls;     // 3T
    std::vector<uint32_t> membrane;  // T: 0 axon (A), 1 myelin (M), 2 glia (G)
    std::vector<uint32_t> fiber;     // T
    uint32_t nAxon = 0, nMyelin = 0, nGlia = 0, nFibers = 0, maxTrianglesOnSurface = 0;
    float maxabs[3] = {1.0f, 1.0f, 1.0f};
};
int parse_mesh_file(const char* path, float spaceScale, MeshHost& out);

// Cylinder file + grid after initFibers(FILE*) and build()/addEntities()
// (dSim2/src/spinSystem.cpp:135-228, 323-385, 483-745)
struct CylHost {
    uint32_t nF = 0;
    std::vector<float> fiberPos;     // 4 per fiber {x, y, z, r^2}; axis coordinate 2.0
    float maxR = 0.0f;
    uint32_t numCubes = 0, maxFPC = 0;
    float cubeLength = 0.0f;
    std::vector<uint32_t> cubeCounter;  // numCubes^3
    std::vector<uint32_t> cubes;        // numCubes^3 * maxFPC
};
int parse_cyl_file(const char* path, float spaceScale, CylHost& out);
int cyl_grid_geometry(CylHost& h);

// sim.cfg subset (libconfig grammar: groups, name = value;, comments) and the
// gradient table (lines of "delta Delta readout Gx Gy Gz")
struct GradRow { float lDelta, bDelta, readOut, gx, gy, gz; };
int parse_grads_file(const char* path, std::vector<GradRow>& rows);

}  // namespace dsim
