// Deterministic scene generation (host only).  The reference builds its scenes in
// mps::System::SurfaceTensionTestScene / ResizeParticle (src/MPS_System/MPSSystem.cpp:357-651)
// and samples its walls from a mesh (src/MPS_Computer/MPSParticleSamplingUtil.cu:42-133); these
// generators emit the same kinds of inputs (jittered lattice blocks, single-layer box walls,
// sampled spheres) directly.  The jitter comes from a counter-based generator (splitmix64 of
// seed and index) evaluated in integer arithmetic, so x86 and Arm produce identical bits.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "mps_c.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Uniform double in [0, 1) from (seed, counter).
inline double uniform01(uint64_t seed, uint64_t counter) {
    const uint64_t r = splitmix64(seed ^ splitmix64(counter));
    return double(r >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace

extern "C" {

int mps_gen_block(int32_t nx, int32_t ny, int32_t nz, const double origin[3], double spacing, double radius,
                  double mass, double jitter, uint64_t seed, float* pos4, float* vel4) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || !origin || !pos4) return MPS_E_INVALID;
    int64_t i = 0;
    for (int32_t z = 0; z < nz; ++z)
        for (int32_t y = 0; y < ny; ++y)
            for (int32_t x = 0; x < nx; ++x, ++i) {
                const int32_t idx[3] = {x, y, z};
                for (int a = 0; a < 3; ++a) {
                    const double u = uniform01(seed, uint64_t(3 * i + a));
                    const double j = jitter * (2.0 * u - 1.0);
                    pos4[4 * i + a] = float(origin[a] + spacing * double(idx[a] + 1) + j);
                }
                pos4[4 * i + 3] = float(radius);
                if (vel4) {
                    vel4[4 * i + 0] = 0.0f;
                    vel4[4 * i + 1] = 0.0f;
                    vel4[4 * i + 2] = 0.0f;
                    vel4[4 * i + 3] = float(mass);
                }
            }
    return MPS_OK;
}

// Lattice points of the box surface; point (i,j,k) is kept when it lies on at least one face
// that is not open.  Per-axis spacing is stretched so that both faces are hit exactly.
int64_t mps_gen_box_walls(const double lo[3], const double hi[3], double spacing, double radius, int32_t open_mask,
                          float* pos4) {
    if (!lo || !hi || !(spacing > 0.0)) return MPS_E_INVALID;
    int64_t n[3];
    double step[3];
    for (int a = 0; a < 3; ++a) {
        const double ext = hi[a] - lo[a];
        if (!(ext > 0.0)) return MPS_E_INVALID;
        n[a] = int64_t(std::llround(ext / spacing)) + 1;
        if (n[a] < 2) n[a] = 2;
        step[a] = ext / double(n[a] - 1);
    }
    int64_t count = 0;
    for (int64_t k = 0; k < n[2]; ++k)
        for (int64_t j = 0; j < n[1]; ++j)
            for (int64_t i = 0; i < n[0]; ++i) {
                const int64_t c[3] = {i, j, k};
                bool on = false;
                for (int a = 0; a < 3 && !on; ++a) {
                    if (c[a] == 0 && !(open_mask & (1 << (2 * a)))) on = true;
                    if (c[a] == n[a] - 1 && !(open_mask & (1 << (2 * a + 1)))) on = true;
                }
                if (!on) continue;
                if (pos4) {
                    for (int a = 0; a < 3; ++a)
                        pos4[4 * count + a] = float(c[a] == n[a] - 1 ? hi[a] : lo[a] + step[a] * double(c[a]));
                    pos4[4 * count + 3] = float(radius);
                }
                count++;
            }
    return count;
}

// Fibonacci lattice on the sphere surface with about one point per spacing^2 of area.
int64_t mps_gen_sphere(const double center[3], double R, double spacing, double radius, float* pos4) {
    if (!center || !(R > 0.0) || !(spacing > 0.0)) return MPS_E_INVALID;
    const double pi = std::acos(-1.0);
    const int64_t count = int64_t(std::llround(4.0 * pi * R * R / (spacing * spacing)));
    if (count <= 0) return 0;
    if (!pos4) return count;
    const double golden = pi * (3.0 - std::sqrt(5.0));
    for (int64_t i = 0; i < count; ++i) {
        const double y = 1.0 - 2.0 * (double(i) + 0.5) / double(count);
        const double r = std::sqrt(std::max(0.0, 1.0 - y * y));
        const double th = golden * double(i);
        pos4[4 * i + 0] = float(center[0] + R * r * std::cos(th));
        pos4[4 * i + 1] = float(center[1] + R * y);
        pos4[4 * i + 2] = float(center[2] + R * r * std::sin(th));
        pos4[4 * i + 3] = float(radius);
    }
    return count;
}

}  // extern "C"
