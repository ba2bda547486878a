// FP64 CPU oracle for the DFSPH step -- TEST INFRASTRUCTURE ONLY (see mps_oracle.h).
//
// Restates moonsh5009/MPS_CUDA's per-frame step with the same operation order per particle
// (neighbour order of the reference's CSR lists, same accumulation order of the fluid and
// boundary partial sums) so that FP64 results agree with the reference's own CUDA step to
// rounding.  Compiled with -ffp-contract=off so that x86 and Arm give identical bits.
// Every function cites the reference file:line it follows (paths inside the reference repo).
#include "mps_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct d3 { double x, y, z; };
inline d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline d3 operator*(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline d3& operator+=(d3& a, d3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline d3& operator-=(d3& a, d3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
inline d3& operator*=(d3& a, double s) { a.x *= s; a.y *= s; a.z *= s; return a; }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double length(d3 a) { return std::sqrt(dot(a, a)); }

// H_RATIO: support radius = 4 x particle radius (src/MPS_Object/MPSDef.h:25-27).
constexpr double kHRatio = 4.0;
const double kPi = std::acos(-1.0);

// Kernel constants written from their formulas (src/MPS_Computer/MPSSPHKernel.cuh:9-15).
struct KConst {
    double w = 315.0 / (64.0 * kPi);       // poly6
    double g = 45.0 / kPi;                 // spiky gradient
    double cw = 8.0 / kPi;                 // cubic spline
    double cg = 48.0 / kPi;                // cubic spline gradient
    double stw = 8.0 / kPi * 10.0 / 7.0 * 2.0;
    double stg = 48.0 / kPi * 10.0 / 7.0;
};
const KConst K;
constexpr double kSphEps = 1.0e-20;
constexpr double kFltEps = 1.1920928955078125e-07;  // FLT_EPSILON = 2^-23

// W(d, 1/h): MPSSPHKernel.cuh:28-45.
inline double WKernel(double dist, double invh, int cubic) {
    const double ratio = dist * invh;
    if (ratio >= 1.0) return 0.0;
    if (cubic) {
        if (ratio >= 0.5) {
            const double t = (1.0 - ratio) * invh;
            return K.cw * 2.0 * t * t * t;
        }
        return K.cw * invh * invh * invh * ((6.0 * ratio - 6.0) * ratio * ratio + 1.0);
    }
    const double t = (1.0 - ratio * ratio) * invh;
    return K.w * t * t * t;
}
// Scalar G with grad W = G * x_ij: MPSSPHKernel.cuh:46-65.
inline double GKernel(double dist, double invh, int cubic) {
    const double ratio = dist * invh;
    if (ratio < kSphEps || ratio >= 1.0) return 0.0;
    const double invh2 = invh * invh;
    if (cubic) {
        if (ratio > 0.5) {
            const double t = (1.0 - ratio) * invh2;
            return -K.cg / dist * t * t;
        }
        return K.cg / dist * invh2 * invh2 * (3.0 * ratio - 2.0) * ratio;
    }
    const double t = (1.0 - ratio) * invh2;
    return -K.g / dist * t * t;
}
// Surface-tension kernels: MPSSPHKernel.cuh:67-84.
inline double STWKernel(double dist, double invh) {
    const double ratio = std::max(dist * invh, 0.5);
    if (ratio >= 1.0) return 0.0;
    const double t = (1.0 - ratio) * invh;
    return K.stw * t * t * t;
}
inline double STGKernel(double dist, double invh) {
    const double ratio = dist * invh;
    if (ratio <= 0.5 || ratio >= 1.0) return 0.0;
    const double t = (1.0 - ratio) * invh * invh;
    return -K.stg / dist * t * t;
}

struct Csr {
    std::vector<uint32_t> idx;  // n+1, inclusive scan with [0]=0
    std::vector<uint32_t> nei;
};

}  // namespace

struct orc_sim {
    orc_params p{};
    int64_t n = 0, nb = 0;
    std::vector<d3> pos, vel, force, grad, predict, cgb;
    std::vector<double> mass, radius, density, alpha, pressure, delta, stfac;
    std::vector<uint32_t> ids;
    std::vector<float> color;
    std::vector<d3> bpos, bvel;
    std::vector<double> bradius, bvol, bmass;
    Csr ff, fb, bb;
    int32_t frame = 0;
    orc_stats st{};
};

namespace {

// ---------------------------------------------------------------- reference hash scheme
// GetGridPos: truncation toward zero plus half the table (MPSSpatialHash.cuh:9-19).
struct I3 { int x, y, z; };
inline I3 grid_pos(d3 x, const uint32_t hs[3], double cell) {
    const double inv = 1.0 / cell;
    return {static_cast<int>(x.x * inv) + static_cast<int>(hs[0] >> 1),
            static_cast<int>(x.y * inv) + static_cast<int>(hs[1] >> 1),
            static_cast<int>(x.z * inv) + static_cast<int>(hs[2] >> 1)};
}
// GetGridIndex: wrapped power-of-two index (MPSSpatialHash.cuh:21-27).
inline uint32_t grid_index(I3 p, const uint32_t hs[3]) {
    return ((static_cast<uint32_t>(p.z) & (hs[2] - 1u)) * hs[1] +
            (static_cast<uint32_t>(p.y) & (hs[1] - 1u))) * hs[0] +
           (static_cast<uint32_t>(p.x) & (hs[0] - 1u));
}
// GetGridZIndex: 10-bit-per-axis Morton code (MPSSpatialHash.cuh:29-45).
inline uint32_t split_by3(uint32_t x) {
    if (x == 1024u) x--;
    x = (x | x << 16u) & 0x030000FFu;
    x = (x | x << 8u) & 0x0300F00Fu;
    x = (x | x << 4u) & 0x030C30C3u;
    x = (x | x << 2u) & 0x09249249u;
    return x;
}
inline uint32_t grid_zindex(I3 p, const uint32_t hs[3]) {
    const uint32_t x = static_cast<uint32_t>(p.x + static_cast<int>(hs[0] >> 1u)) & (hs[0] - 1u);
    const uint32_t y = static_cast<uint32_t>(p.y + static_cast<int>(hs[1] >> 1u)) & (hs[1] - 1u);
    const uint32_t z = static_cast<uint32_t>(p.z + static_cast<int>(hs[2] >> 1u)) & (hs[2] - 1u);
    return split_by3(x) | (split_by3(y) << 1u) | (split_by3(z) << 2u);
}

struct Hash {
    std::vector<uint32_t> key, id, start, end;
};

// UpdateHash: keys, stable sort by key, start/end by adjacent difference
// (MPSSpatialHash.cu:53-77, MPSSpatialHash.cuh:83-98,115-145).
void update_hash(Hash& h, const std::vector<d3>& pos, const orc_params& p) {
    const size_t n = pos.size();
    const size_t cells = size_t(p.hash_size[0]) * p.hash_size[1] * p.hash_size[2];
    h.start.assign(cells, 0xffffffffu);
    h.end.assign(cells, 0xffffffffu);
    h.key.resize(n);
    h.id.resize(n);
    for (size_t i = 0; i < n; ++i) {
        h.key[i] = grid_index(grid_pos(pos[i], p.hash_size, p.hash_cell), p.hash_size);
        h.id[i] = uint32_t(i);
    }
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return h.key[a] < h.key[b]; });
    std::vector<uint32_t> k2(n), i2(n);
    for (size_t i = 0; i < n; ++i) { k2[i] = h.key[order[i]]; i2[i] = h.id[order[i]]; }
    h.key.swap(k2);
    h.id.swap(i2);
    for (size_t i = 0; i < n; ++i) {
        const uint32_t k = h.key[i];
        if (i == 0 || h.key[i - 1] != k) {
            h.start[k] = uint32_t(i);
            if (i > 0) h.end[h.key[i - 1]] = uint32_t(i);
        }
        if (i == n - 1) h.end[k] = uint32_t(n);
    }
}

// Research: 27-cell loop z, y, x (MPSSpatialHash.cuh:47-80); criterion
// |xi - xj| < (hi + hj) / 2 with h = 4 r, self excluded for the same set
// (ComputeNeighborhoodSize_kernel / BuildNeighborhood_kernel, MPSSpatialHash.cuh:147-271).
void build_csr(Csr& out, const std::vector<d3>& q, const std::vector<double>& qr,
               const std::vector<d3>& ref, const std::vector<double>& rr, const Hash& h,
               const orc_params& p, bool same) {
    const int64_t n = int64_t(q.size());
    std::vector<std::vector<uint32_t>> lists(static_cast<size_t>(n));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const d3 xi = q[size_t(i)];
        const double ri = qr[size_t(i)] * kHRatio;
        const I3 c = grid_pos(xi, p.hash_size, p.hash_cell);
        auto& L = lists[size_t(i)];
        I3 g;
        for (g.z = c.z - 1; g.z <= c.z + 1; g.z++)
            for (g.y = c.y - 1; g.y <= c.y + 1; g.y++)
                for (g.x = c.x - 1; g.x <= c.x + 1; g.x++) {
                    const uint32_t cell = grid_index(g, p.hash_size);
                    uint32_t s = h.start[cell];
                    const uint32_t e = h.end[cell];
                    for (; s < e; s++) {
                        const uint32_t jd = h.id[s];
                        if (same && jd == uint32_t(i)) continue;
                        const double rj = rr[jd] * kHRatio;
                        const double dist = length(xi - ref[jd]);
                        if (dist < (ri + rj) * 0.5) L.push_back(jd);
                    }
                }
    }
    out.idx.assign(size_t(n) + 1, 0u);
    for (int64_t i = 0; i < n; ++i) out.idx[size_t(i) + 1] = out.idx[size_t(i)] + uint32_t(lists[size_t(i)].size());
    out.nei.resize(out.idx[size_t(n)]);
    for (int64_t i = 0; i < n; ++i)
        std::copy(lists[size_t(i)].begin(), lists[size_t(i)].end(), out.nei.begin() + out.idx[size_t(i)]);
}

template <class Fn>
inline void for_nei(const Csr& c, int64_t i, Fn fn) {
    for (uint32_t k = c.idx[size_t(i)]; k < c.idx[size_t(i) + 1]; ++k) fn(c.nei[k]);
}

double seq_sum(const std::vector<double>& v) {
    double s = 0.0;
    for (double x : v) s += x;
    return s;
}

// ------------------------------------------------------------------------- phases
// ZSort of fluid and boundary: Morton key then stable sort of the zipped arrays
// (MPSSpatialHash.cu:79-140).  The boundary volume is NOT permuted (D11 quirk, :124-140).
void phase_zsort(orc_sim& s) {
    if (!s.p.zsort || (s.frame % 50) != 1) return;
    auto perm_of = [&](const std::vector<d3>& pos) {
        std::vector<uint32_t> key(pos.size());
        for (size_t i = 0; i < pos.size(); ++i)
            key[i] = grid_zindex(grid_pos(pos[i], s.p.hash_size, s.p.hash_cell), s.p.hash_size);
        std::vector<uint32_t> order(pos.size());
        std::iota(order.begin(), order.end(), 0u);
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
        return order;
    };
    auto apply = [](auto& v, const std::vector<uint32_t>& o) {
        auto t = v;
        for (size_t i = 0; i < o.size(); ++i) v[i] = t[o[i]];
    };
    if (s.nb) {
        const auto o = perm_of(s.bpos);
        apply(s.bpos, o); apply(s.bmass, o); apply(s.bvel, o); apply(s.bradius, o);
    }
    if (s.n) {
        const auto o = perm_of(s.pos);
        apply(s.pos, o); apply(s.mass, o); apply(s.vel, o); apply(s.radius, o); apply(s.ids, o);
        std::vector<float> c = s.color;
        for (size_t i = 0; i < o.size(); ++i)
            for (int k = 0; k < 4; ++k) s.color[4 * i + k] = c[4 * size_t(o[i]) + k];
    }
}

// UpdateHash x2 + BuildNeighorhood x3 (MPSSystem.cpp:226-235).
void phase_neighbors(orc_sim& s) {
    Hash hb, hf;
    if (s.nb) update_hash(hb, s.bpos, s.p);
    if (s.n) update_hash(hf, s.pos, s.p);
    s.bb = Csr{}; s.ff = Csr{}; s.fb = Csr{};
    if (s.nb) build_csr(s.bb, s.bpos, s.bradius, s.bpos, s.bradius, hb, s.p, true);
    if (s.n) build_csr(s.ff, s.pos, s.radius, s.pos, s.radius, hf, s.p, true);
    if (s.n && s.nb) build_csr(s.fb, s.pos, s.radius, s.bpos, s.bradius, hb, s.p, false);
    if (s.n && !s.nb) s.fb.idx.assign(size_t(s.n) + 1, 0u);
    s.st.nei_ff = s.ff.nei.size();
    s.st.nei_fb = s.fb.nei.size();
    s.st.nei_bb = s.bb.nei.size();
}

// ComputeBoundaryParticleVolumeSub/Final (MPSSPHBaseUtil.cuh:10-41,78-86).  The reference
// accumulates onto the previous value (no reset, MPSSystem.cpp:237-238).
void phase_bvolume(orc_sim& s) {
    const int64_t nb = s.nb;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nb; ++i) {
        const double hi = s.bradius[size_t(i)] * kHRatio;
        const double invHi = 1.0 / hi;
        const d3 xi = s.bpos[size_t(i)];
        double volume = WKernel(0.0, invHi, s.p.cubic);
        for_nei(s.bb, i, [&](uint32_t jd) { volume += WKernel(length(xi - s.bpos[jd]), invHi, s.p.cubic); });
        const double prev = s.p.volume_accumulate ? s.bvol[size_t(i)] : 0.0;
        s.bvol[size_t(i)] = 1.0 / (prev + volume);
    }
}

// ResetREAL + ComputeDensitySub(fluid) + ComputeDensitySub(boundary) + Final + colour
// (MPSSystem.cpp:240-245; MPSSPHBaseUtil.cuh:88-120,158-221).
void phase_density(orc_sim& s) {
    const int64_t n = s.n;
    const double V = s.p.mat_volume;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double hi = s.radius[size_t(i)] * kHRatio;
        const double invHi = 1.0 / hi;
        const d3 xi = s.pos[size_t(i)];
        double df = V * WKernel(0.0, invHi, s.p.cubic);
        for_nei(s.ff, i, [&](uint32_t jd) { df += V * WKernel(length(xi - s.pos[jd]), invHi, s.p.cubic); });
        double db = 0.0;
        for_nei(s.fb, i, [&](uint32_t jd) { db += s.bvol[jd] * WKernel(length(xi - s.bpos[jd]), invHi, s.p.cubic); });
        const double rho = ((0.0 + df) + db) * s.p.mat_density;
        s.density[size_t(i)] = rho;
        const float ratio = static_cast<float>(rho / s.p.mat_density);
        auto clampf = [](float v) { return std::min(std::max(v, 0.0f), 1.0f); };
        s.color[4 * size_t(i) + 0] = clampf(ratio - 1.0f);
        s.color[4 * size_t(i) + 1] = clampf(ratio < 1.0f ? ratio : 1.0f - (ratio - 1.0f));
        s.color[4 * size_t(i) + 2] = clampf(1.0f - ratio);
        s.color[4 * size_t(i) + 3] = 1.0f;
    }
}

// ComputeDFSPHFactorSub x2 + Final (MPSSystem.cpp:247-251; MPSSPHDFSPHUtil.cuh:10-47,90-137).
void phase_alpha(orc_sim& s) {
    const int64_t n = s.n;
    const double V = s.p.mat_volume;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double hi = s.radius[size_t(i)] * kHRatio;
        const double invHi = 1.0 / hi;
        const d3 xi = s.pos[size_t(i)];
        d3 grads{0, 0, 0};
        double fac = 0.0;
        for_nei(s.ff, i, [&](uint32_t jd) {
            const d3 xij = xi - s.pos[jd];
            const d3 g = (V * GKernel(length(xij), invHi, s.p.cubic)) * xij;
            grads += g;
            fac += dot(g, g);
        });
        d3 gb{0, 0, 0};
        for_nei(s.fb, i, [&](uint32_t jd) {
            const d3 xij = xi - s.bpos[jd];
            gb += (s.bvol[jd] * GKernel(length(xij), invHi, s.p.cubic)) * xij;
        });
        const d3 gs = (d3{0, 0, 0} + grads) + gb;
        s.grad[size_t(i)] = gs;
        double f = (0.0 + fac) + dot(gs, gs);
        s.alpha[size_t(i)] = f > kSphEps ? 1.0 / f : 0.0;
    }
}

// UpdateVelocity: v += dt / m * F when m > 1e-10 (MPSAdvectUtil.cuh:20-34).
void update_velocity(orc_sim& s) {
    const int64_t n = s.n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        if (s.mass[size_t(i)] > 1.0e-10)
            s.vel[size_t(i)] += (s.p.dt / s.mass[size_t(i)]) * s.force[size_t(i)];
}

// ResetForce, ApplyGravity, UpdateVelocity (MPSSystem.cpp:253-255; MPSAdvectUtil.cuh:8-18).
void phase_gravity(orc_sim& s) {
    const d3 g{s.p.gravity[0], s.p.gravity[1], s.p.gravity[2]};
    for (int64_t i = 0; i < s.n; ++i) s.force[size_t(i)] = d3{0, 0, 0} + g * s.mass[size_t(i)];
    update_velocity(s);
}

// ComputeDensityDelta_kernel fluid + boundary (MPSSPHDFSPHUtil.cuh:139-175,218-257).
void density_delta(orc_sim& s) {
    const int64_t n = s.n;
    const double V = s.p.mat_volume;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double invHi = 1.0 / (s.radius[size_t(i)] * kHRatio);
        const d3 xi = s.pos[size_t(i)], vi = s.vel[size_t(i)];
        double df = 0.0, db = 0.0;
        for_nei(s.ff, i, [&](uint32_t jd) {
            const d3 xij = xi - s.pos[jd], vij = vi - s.vel[jd];
            df += V * GKernel(length(xij), invHi, s.p.cubic) * dot(xij, vij);
        });
        for_nei(s.fb, i, [&](uint32_t jd) {
            const d3 xij = xi - s.bpos[jd], vij = vi - s.bvel[jd];
            db += s.bvol[jd] * GKernel(length(xij), invHi, s.p.cubic) * dot(xij, vij);
        });
        s.delta[size_t(i)] = (0.0 + df) + db;
    }
}

// ApplyDFSPH_kernel fluid + boundary + Final, then UpdateVelocity
// (MPSSPHDFSPHUtil.cuh:342-377,420-468; MPSSPHDFSPHUtil.cu:427-431).
void apply_pressure(orc_sim& s) {
    const int64_t n = s.n;
    const double V = s.p.mat_volume;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double invHi = 1.0 / (s.radius[size_t(i)] * kHRatio);
        const d3 xi = s.pos[size_t(i)];
        const double pi = s.pressure[size_t(i)];
        d3 ff{0, 0, 0}, fb{0, 0, 0};
        for_nei(s.ff, i, [&](uint32_t jd) {
            const d3 xij = xi - s.pos[jd];
            ff -= (0.5 * V * (pi + s.pressure[jd]) * GKernel(length(xij), invHi, s.p.cubic)) * xij;
        });
        for_nei(s.fb, i, [&](uint32_t jd) {
            const d3 xij = xi - s.bpos[jd];
            fb -= (0.5 * s.bvol[jd] * pi * GKernel(length(xij), invHi, s.p.cubic)) * xij;
        });
        s.force[size_t(i)] = s.mass[size_t(i)] * ((d3{0, 0, 0} + ff) + fb);
    }
    update_velocity(s);
}

// Shared solver loop of ComputeDFSPHDivergenceFree (MPSSPHDFSPHUtil.cu:385-441) and
// ComputeDFSPHConstantDensity (:270-384); stiffness rules from MPSSPHDFSPHUtil.cuh:259-340.
int pressure_solve(orc_sim& s, bool divergence, double* err_out) {
    const int64_t n = s.n;
    if (n == 0) return 0;
    const double dt = s.p.dt;
    const double tol = divergence ? s.p.df_tol : s.p.cd_tol;
    const int minl = divergence ? s.p.df_min_iter : s.p.cd_min_iter;
    std::vector<double> errs(static_cast<size_t>(n));
    int l = 1;
    double err = 0.0;
    const int cap = s.p.fixed_iters > 0 ? s.p.fixed_iters : s.p.max_iter;
    while (l <= cap) {
        density_delta(s);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            const double r = s.density[size_t(i)] / s.p.mat_density;
            const double d = s.delta[size_t(i)];
            double k = divergence ? std::min(d * dt, r + dt * d - 0.8) : r + dt * d - 1.0;
            errs[size_t(i)] = 0.0;
            if (k > 0.0) {
                errs[size_t(i)] = k;
                k *= s.alpha[size_t(i)] / (dt * dt);
            } else {
                k = 0.0;
            }
            s.pressure[size_t(i)] = k;
        }
        err = seq_sum(errs) / double(n);
        if (s.p.fixed_iters > 0 ? l > s.p.fixed_iters : (err < tol && l > minl)) break;
        apply_pressure(s);
        l++;
        if (s.p.fixed_iters > 0 && l > s.p.fixed_iters) break;
    }
    *err_out = err;
    return l;
}

// ComputeSurfaceTensionFactor_kernel (MPSSPHNonPressureUtil.cuh:425-465).
void st_factor(orc_sim& s) {
    const int64_t n = s.n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double invHi = 1.0 / (s.radius[size_t(i)] * kHRatio);
        const d3 xi = s.pos[size_t(i)], vi = s.vel[size_t(i)];
        double d = 0.0;
        for_nei(s.ff, i, [&](uint32_t jd) {
            const d3 xij = xi - s.pos[jd], vij = vi - s.vel[jd];
            const d3 g = GKernel(length(xij), invHi, s.p.cubic) * xij;
            d += s.mass[jd] * dot(vij, g);
        });
        s.stfac[size_t(i)] = d;
    }
}

// g_ij of the surface-tension terms (MPSSPHNonPressureUtil.cuh:510-515, :570-575).
inline double st_gij(const orc_sim& s, int64_t i, uint32_t jd, d3 xij, double dist, double invHi) {
    const d3 vij = s.vel[size_t(i)] - s.vel[jd];
    const double invDij = 2.0 / (s.density[size_t(i)] + s.density[jd]);
    const double stW = STWKernel(dist, invHi);
    const d3 stG = STGKernel(dist, invHi) * xij;
    return (stW + s.p.dt * (dot(vij, stG) - (s.stfac[size_t(i)] + s.stfac[jd]) * invDij * 0.5 * stW)) * invDij;
}

// ComputeSurfaceTensionCGb_kernel (MPSSPHNonPressureUtil.cuh:467-521).
void st_cgb(orc_sim& s) {
    const int64_t n = s.n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double invHi = 1.0 / (s.radius[size_t(i)] * kHRatio);
        const d3 xi = s.pos[size_t(i)];
        const double mi = s.mass[size_t(i)];
        d3 bi{0, 0, 0};
        for_nei(s.ff, i, [&](uint32_t jd) {
            const d3 xij = xi - s.pos[jd];
            const double dist = length(xij);
            const double mij = 0.5 * (mi + s.mass[jd]);
            bi -= (mij * st_gij(s, i, jd, xij, dist, invHi)) * xij;
        });
        s.cgb[size_t(i)] = (s.p.dt * s.p.surface_tension / mi) * bi + s.vel[size_t(i)];
    }
}

// A p = p (1 + f) + dt (ST + XSPH + viscosity) over fluid neighbours
// (ComputeSurfaceTensionCGAp_kernel :523-585, ComputeCGViscosityAp_kernel :587-635,
//  ComputeFinalCGAp_kernel :637-648 of MPSSPHNonPressureUtil.cuh).
void cg_apply(const orc_sim& s, const std::vector<d3>& p, std::vector<d3>& Ap, double factor) {
    const int64_t n = s.n;
    const double dt = s.p.dt;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double hi = s.radius[size_t(i)] * kHRatio;
        const double invHi = 1.0 / hi;
        const d3 xi = s.pos[size_t(i)], pi = p[size_t(i)];
        const double mi = s.mass[size_t(i)], di = s.density[size_t(i)];
        d3 apst{0, 0, 0}, apx{0, 0, 0};
        for_nei(s.ff, i, [&](uint32_t jd) {
            const d3 xij = xi - s.pos[jd];
            const double dist = length(xij);
            const double mij = 0.5 * (mi + s.mass[jd]);
            const double gij = st_gij(s, i, jd, xij, dist, invHi);
            const d3 pij = pi - p[jd];
            apst += (mij * gij) * pij;
            apx += (s.mass[jd] / s.density[jd]) * pij * WKernel(dist, invHi, s.p.cubic);
        });
        apst *= dt * s.p.surface_tension / mi;
        apx *= s.p.xsph / dt;
        d3 av{0, 0, 0};
        for_nei(s.ff, i, [&](uint32_t jd) {
            const double onePercentHSq = 0.01 * hi * hi;
            const d3 xij = xi - s.pos[jd];
            const d3 pij = pi - p[jd];
            const double dist = length(xij);
            const d3 dp = (0.5 * (mi + s.mass[jd]) / s.density[jd] * dot(pij, xij) /
                           (dist * dist + onePercentHSq) * GKernel(dist, invHi, s.p.cubic) /
                           (dist + kFltEps)) * xij;
            av -= dp;
        });
        av *= 10.0 * s.p.mat_density * s.p.viscosity / di;
        const d3 acc = (d3{0, 0, 0} + (apst + apx)) + av;
        Ap[size_t(i)] = pi * (1.0 + factor) + dt * acc;
    }
}

double dot3n(const std::vector<d3>& a, const std::vector<d3>& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) {
        s += a[i].x * b[i].x;
        s += a[i].y * b[i].y;
        s += a[i].z * b[i].z;
    }
    return s;
}

// 3x3 diagonal block of A_0 + f I per particle (symmetric):
// (1 + f) I + dt [sum_j (ST + XSPH coefficient) I - sum_j (viscosity coefficient) x_ij x_ij^T],
// the coefficients of cg_apply's terms; returned inverted (6 entries xx, yy, zz, xy, xz, yz).
// A block with a non-positive or non-finite determinant is replaced by (1 + f) I.
struct Sym3 {
    double xx, yy, zz, xy, xz, yz;
};
Sym3 sym3_inverse(const Sym3& a, double fallback, bool* ok) {
    const double c00 = a.yy * a.zz - a.yz * a.yz;
    const double c01 = a.xz * a.yz - a.xy * a.zz;
    const double c02 = a.xy * a.yz - a.xz * a.yy;
    const double det = a.xx * c00 + a.xy * c01 + a.xz * c02;
    if (!(det > 1.0e-30) || !std::isfinite(det)) {
        *ok = false;
        return Sym3{1.0 / fallback, 1.0 / fallback, 1.0 / fallback, 0.0, 0.0, 0.0};
    }
    *ok = true;
    const double id = 1.0 / det;
    return Sym3{c00 * id, (a.xx * a.zz - a.xz * a.xz) * id, (a.xx * a.yy - a.xy * a.xy) * id, c01 * id, c02 * id,
                (a.xy * a.xz - a.xx * a.yz) * id};
}
inline d3 sym3_mul(const Sym3& m, d3 v) {
    return d3{m.xx * v.x + m.xy * v.y + m.xz * v.z, m.xy * v.x + m.yy * v.y + m.yz * v.z,
              m.xz * v.x + m.yz * v.y + m.zz * v.z};
}

void jacobi_blocks(const orc_sim& s, std::vector<Sym3>& Dinv, double factor) {
    const int64_t n = s.n;
    const double dt = s.p.dt;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double hi = s.radius[size_t(i)] * kHRatio;
        const double invHi = 1.0 / hi;
        const d3 xi = s.pos[size_t(i)];
        const double mi = s.mass[size_t(i)], di = s.density[size_t(i)];
        double cst = 0.0, cx = 0.0;
        Sym3 cv{0, 0, 0, 0, 0, 0};
        for_nei(s.ff, i, [&](uint32_t jd) {
            const d3 xij = xi - s.pos[jd];
            const double dist = length(xij);
            const double mij = 0.5 * (mi + s.mass[jd]);
            cst += mij * st_gij(s, i, jd, xij, dist, invHi);
            cx += (s.mass[jd] / s.density[jd]) * WKernel(dist, invHi, s.p.cubic);
            const double c = 0.5 * (mi + s.mass[jd]) / s.density[jd] / (dist * dist + 0.01 * hi * hi) *
                             GKernel(dist, invHi, s.p.cubic) / (dist + kFltEps);
            cv.xx += c * xij.x * xij.x; cv.yy += c * xij.y * xij.y; cv.zz += c * xij.z * xij.z;
            cv.xy += c * xij.x * xij.y; cv.xz += c * xij.x * xij.z; cv.yz += c * xij.y * xij.z;
        });
        const double c0 = (dt * s.p.surface_tension / mi) * cst + (s.p.xsph / dt) * cx;
        const double vs = 10.0 * s.p.mat_density * s.p.viscosity / di;
        const double dg = (1.0 + factor) + dt * c0;
        const Sym3 D{dg - dt * vs * cv.xx, dg - dt * vs * cv.yy, dg - dt * vs * cv.zz, -dt * vs * cv.xy,
                     -dt * vs * cv.xz, -dt * vs * cv.yz};
        bool ok;
        Dinv[size_t(i)] = sym3_inverse(D, 1.0 + factor, &ok);
    }
}

// Block-Jacobi alternative of the CG on the same system: from x0 = v,
// x += D^-1 (b + f x0 - (A_0 + f I) x), D = the 3x3 diagonal blocks, until r.r < cg_tol (at most
// cg_max_iter sweeps) or for fixed_iters sweeps (the reference's legacy Jacobi viscosity,
// MPSSPHNonPressureUtil.cuh:90-195, also inverted each particle's 3x3 block, there of the
// viscosity term alone).
int viscst_jacobi(orc_sim& s, double* rr_out) {
    const int64_t n = s.n;
    const double f = 0.01;   // the CG iterations' operator factor (MPSSPHNonPressureUtil.cu:165-169)
    std::vector<Sym3> Dinv(static_cast<size_t>(n));
    std::vector<d3> Ax(static_cast<size_t>(n));
    jacobi_blocks(s, Dinv, f);
    std::vector<d3>& x = s.predict;
    const std::vector<d3> x0 = s.vel;
    int l = 1;
    const int cap = s.p.fixed_iters > 0 ? s.p.fixed_iters : s.p.cg_max_iter;
    while (l <= cap) {
        cg_apply(s, x, Ax, f);
        double rr = 0.0;
        std::vector<d3> r(static_cast<size_t>(n));
        for (int64_t i = 0; i < n; ++i) {
            r[size_t(i)] = (s.cgb[size_t(i)] + f * x0[size_t(i)]) - Ax[size_t(i)];
            rr += r[size_t(i)].x * r[size_t(i)].x;
            rr += r[size_t(i)].y * r[size_t(i)].y;
            rr += r[size_t(i)].z * r[size_t(i)].z;
        }
        *rr_out = rr;
        if (s.p.fixed_iters <= 0 && rr < s.p.cg_tol) break;
        for (int64_t i = 0; i < n; ++i) x[size_t(i)] += sym3_mul(Dinv[size_t(i)], r[size_t(i)]);
        l++;
    }
    return l;
}

// ApplyImplicitViscosityNSurfaceTension + CGSolver (MPSSPHNonPressureUtil.cu:127-188,
// MPSSolver.cuh:12-73, MPSCGKernel.cuh:5-133).  The operator uses f = 0 for A x0 and
// f = 0.01 for every iteration (:165-169).
int phase_viscst(orc_sim& s, double* rr_out) {
    const int64_t n = s.n;
    *rr_out = 0.0;
    if (n == 0) return 0;
    s.predict = s.vel;
    st_factor(s);
    st_cgb(s);
    if (s.p.visc_solver == 1) {
        const int l = viscst_jacobi(s, rr_out);
        s.vel = s.predict;
        return l;
    }
    std::vector<d3> r(static_cast<size_t>(n)), p(static_cast<size_t>(n)), Ap(static_cast<size_t>(n));
    std::vector<d3>& x = s.predict;
    cg_apply(s, x, Ap, 0.0);
    for (int64_t i = 0; i < n; ++i) { r[size_t(i)] = s.cgb[size_t(i)] - Ap[size_t(i)]; p[size_t(i)] = r[size_t(i)]; }
    int l = 1;
    const int cap = s.p.fixed_iters > 0 ? s.p.fixed_iters : s.p.cg_max_iter;
    while (l <= cap) {
        cg_apply(s, p, Ap, 0.01);
        const double rr = dot3n(r, r), pAp = dot3n(p, Ap);
        *rr_out = rr;
        if (s.p.fixed_iters <= 0 && rr < s.p.cg_tol) break;
        const double a = rr / pAp;
        for (int64_t i = 0; i < n; ++i) {
            x[size_t(i)] = x[size_t(i)] + a * p[size_t(i)];
            r[size_t(i)] = r[size_t(i)] - a * Ap[size_t(i)];
        }
        const double rr2 = dot3n(r, r);
        const double b = rr2 / rr;
        for (int64_t i = 0; i < n; ++i) p[size_t(i)] = r[size_t(i)] + b * p[size_t(i)];
        l++;
    }
    s.vel = s.predict;
    return l;
}

// BoundaryCollision then UpdatePosition (MPSAdvectUtil.cuh:36-77).
void phase_advect(orc_sim& s) {
    const double dt = s.p.dt;
    auto axis = [](double pos, double lo, double hi, double v) {
        if (pos < lo && v < 0.0) return std::fabs(v) < 1.0e-4 ? 0.0 : -v * 0.4;
        if (pos > hi && v > 0.0) return std::fabs(v) < 1.0e-4 ? 0.0 : -v * 0.4;
        return v;
    };
    for (int64_t i = 0; i < s.n; ++i) {
        d3 v = s.vel[size_t(i)];
        const d3 x = s.pos[size_t(i)] + v * dt;
        v.x = axis(x.x, s.p.bmin[0], s.p.bmax[0], v.x);
        v.y = axis(x.y, s.p.bmin[1], s.p.bmax[1], v.y);
        v.z = axis(x.z, s.p.bmin[2], s.p.bmax[2], v.z);
        s.vel[size_t(i)] = v;
        s.pos[size_t(i)] += dt * v;
    }
    s.frame++;
    s.st.frame = s.frame;
}

template <class T>
int64_t copy_out(const std::vector<T>& v, void* out) {
    if (out) std::memcpy(out, v.data(), v.size() * sizeof(T));
    return int64_t(v.size());
}
int64_t copy_out3(const std::vector<d3>& v, void* out) {
    if (out) std::memcpy(out, v.data(), v.size() * sizeof(d3));
    return int64_t(v.size() * 3);
}

}  // namespace

extern "C" {

orc_sim* orc_create(const orc_params* p) {
    auto* s = new orc_sim();
    s->p = *p;
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
    return s;
}

void orc_destroy(orc_sim* s) { delete s; }

// Replaces the parameters (tolerances, iteration caps, fixed_iters, ...) of a live replay; the
// precision study reruns one solve with another iteration count from the same state.
void orc_set_params(orc_sim* s, const orc_params* p) {
    s->p = *p;
#ifdef _OPENMP
    if (p->threads > 0) omp_set_num_threads(p->threads);
#endif
}

int orc_set_fluid(orc_sim* s, int64_t n, const double* pos, const double* vel, const double* mass,
                  const double* radius, const uint32_t* ids) {
    if (n < 0) return -1;
    s->n = n;
    const size_t un = size_t(n);
    s->pos.assign(reinterpret_cast<const d3*>(pos), reinterpret_cast<const d3*>(pos) + un);
    s->vel.assign(reinterpret_cast<const d3*>(vel), reinterpret_cast<const d3*>(vel) + un);
    s->mass.assign(mass, mass + un);
    s->radius.assign(radius, radius + un);
    s->ids.resize(un);
    for (size_t i = 0; i < un; ++i) s->ids[i] = ids ? ids[i] : uint32_t(i);
    s->force.assign(un, d3{0, 0, 0});
    s->grad.assign(un, d3{0, 0, 0});
    s->predict.assign(un, d3{0, 0, 0});
    s->cgb.assign(un, d3{0, 0, 0});
    s->density.assign(un, 0.0);
    s->alpha.assign(un, 0.0);
    s->pressure.assign(un, 0.0);
    s->delta.assign(un, 0.0);
    s->stfac.assign(un, 0.0);
    s->color.assign(4 * un, 0.0f);
    return 0;
}

int orc_set_boundary(orc_sim* s, int64_t nb, const double* pos, const double* radius, const double* volume) {
    if (nb < 0) return -1;
    s->nb = nb;
    const size_t un = size_t(nb);
    s->bpos.assign(reinterpret_cast<const d3*>(pos), reinterpret_cast<const d3*>(pos) + un);
    s->bradius.assign(radius, radius + un);
    s->bvol.assign(un, 0.0);
    if (volume) s->bvol.assign(volume, volume + un);
    s->bvel.assign(un, d3{0, 0, 0});
    s->bmass.assign(un, 0.0);
    return 0;
}

void orc_set_frame(orc_sim* s, int32_t frame) { s->frame = frame; s->st.frame = frame; }

int orc_phase(orc_sim* s, int32_t phase) {
    switch (phase) {
        case ORC_ZSORT: phase_zsort(*s); break;
        case ORC_NEIGHBORS: phase_neighbors(*s); break;
        case ORC_BVOLUME: phase_bvolume(*s); break;
        case ORC_DENSITY: phase_density(*s); break;
        case ORC_ALPHA: phase_alpha(*s); break;
        case ORC_GRAVITY: phase_gravity(*s); break;
        case ORC_DF: s->st.df_iters = pressure_solve(*s, true, &s->st.df_err); break;
        case ORC_VISCST: s->st.cg_iters = phase_viscst(*s, &s->st.cg_rr); break;
        case ORC_CD: s->st.cd_iters = pressure_solve(*s, false, &s->st.cd_err); break;
        case ORC_ADVECT: phase_advect(*s); break;
        default: return -1;
    }
    return 0;
}

int orc_step(orc_sim* s, int32_t nsteps) {
    for (int k = 0; k < nsteps; ++k)
        for (int ph = ORC_ZSORT; ph <= ORC_ADVECT; ++ph) orc_phase(s, ph);
    return 0;
}

void orc_get_stats(const orc_sim* s, orc_stats* out) { *out = s->st; }

int64_t orc_get(const orc_sim* s, const char* name, void* out) {
    const std::string k(name);
    if (k == "pos") return copy_out3(s->pos, out);
    if (k == "vel") return copy_out3(s->vel, out);
    if (k == "force") return copy_out3(s->force, out);
    if (k == "gradsum") return copy_out3(s->grad, out);
    if (k == "cg_b") return copy_out3(s->cgb, out);
    if (k == "mass") return copy_out(s->mass, out);
    if (k == "radius") return copy_out(s->radius, out);
    if (k == "ids") return copy_out(s->ids, out);
    if (k == "density") return copy_out(s->density, out);
    if (k == "alpha") return copy_out(s->alpha, out);
    if (k == "pressure") return copy_out(s->pressure, out);
    if (k == "delta") return copy_out(s->delta, out);
    if (k == "stfac") return copy_out(s->stfac, out);
    if (k == "color") return copy_out(s->color, out);
    if (k == "bpos") return copy_out3(s->bpos, out);
    if (k == "bradius") return copy_out(s->bradius, out);
    if (k == "bvol") return copy_out(s->bvol, out);
    if (k == "nei_ff_idx") return copy_out(s->ff.idx, out);
    if (k == "nei_fb_idx") return copy_out(s->fb.idx, out);
    if (k == "nei_bb_idx") return copy_out(s->bb.idx, out);
    if (k == "nei_ff") return copy_out(s->ff.nei, out);
    if (k == "nei_fb") return copy_out(s->fb.nei, out);
    if (k == "nei_bb") return copy_out(s->bb.nei, out);
    return -1;
}

int orc_put(orc_sim* s, const char* name, const void* in, int64_t count) {
    const std::string k(name);
    auto put = [&](std::vector<double>& v, int64_t expect) {
        if (count != expect) return -1;
        std::memcpy(v.data(), in, size_t(count) * sizeof(double));
        return 0;
    };
    if (k == "vel") { if (count != 3 * s->n) return -1; std::memcpy(s->vel.data(), in, size_t(count) * 8); return 0; }
    if (k == "pos") { if (count != 3 * s->n) return -1; std::memcpy(s->pos.data(), in, size_t(count) * 8); return 0; }
    if (k == "density") return put(s->density, s->n);
    if (k == "alpha") return put(s->alpha, s->n);
    if (k == "pressure") return put(s->pressure, s->n);
    if (k == "stfac") return put(s->stfac, s->n);
    if (k == "bvol") return put(s->bvol, s->nb);
    return -1;
}

// ------------------------------------------------------------------ new integer scheme
static inline int cell_coord(float x, float o, float inv, int dim) {
    const float t = (x - o) * inv;
    if (!(t >= 0.0f)) return 0;           // negative or NaN
    if (t >= float(dim)) return dim - 1;
    const int c = int(t);
    return c < dim ? c : dim - 1;
}

// Key of cell (cx, cy, cz): cells grouped in columns of 2 x 2 rows (y, z) along x; inside a
// column the key runs over x, then over the column's 4 rows (y fastest); ny and nz are padded to
// even counts.  The GPU step's key layout (grid_key of the CUDA library), restated.
static inline uint64_t new_key(const orc_grid* g, int cx, int cy, int cz) {
    const uint64_t nyb = (uint64_t(g->dims[1]) + 1) / 2;
    const uint64_t col = uint64_t(cz / 2) * nyb + uint64_t(cy / 2);
    return g->key_base + ((col * uint64_t(g->dims[0]) + uint64_t(cx)) * 2 + uint64_t(cz % 2)) * 2 + uint64_t(cy % 2);
}

void orc_new_keys(int64_t n, const float* pos4, const orc_grid* g, uint64_t* keys) {
    for (int64_t i = 0; i < n; ++i) {
        const float* p = pos4 + 4 * i;
        const int cx = cell_coord(p[0], g->origin[0], g->inv_cell, g->dims[0]);
        const int cy = cell_coord(p[1], g->origin[1], g->inv_cell, g->dims[1]);
        const int cz = cell_coord(p[2], g->origin[2], g->inv_cell, g->dims[2]);
        keys[i] = new_key(g, cx, cy, cz);
    }
}

void orc_new_stable_sort(int64_t n, uint64_t* keys, uint32_t* vals) {
    std::vector<uint32_t> o(static_cast<size_t>(n));
    std::iota(o.begin(), o.end(), 0u);
    std::stable_sort(o.begin(), o.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    std::vector<uint64_t> k(keys, keys + n);
    std::vector<uint32_t> v(vals, vals + n);
    for (int64_t i = 0; i < n; ++i) { keys[i] = k[o[size_t(i)]]; vals[i] = v[o[size_t(i)]]; }
}

int64_t orc_new_cell_ranges(int64_t n, const uint64_t* sk, uint64_t* cells, uint32_t* starts, uint32_t* ends) {
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (i == 0 || sk[i] != sk[i - 1]) {
            cells[m] = sk[i];
            starts[m] = uint32_t(i);
            if (m > 0) ends[m - 1] = uint32_t(i);
            m++;
        }
    }
    if (m > 0) ends[m - 1] = uint32_t(n);
    return m;
}

void orc_new_nbr_counts(int64_t nq, const float* q4, int64_t np, const float* p4, const uint64_t* psk,
                        const orc_grid* g, int same_set, uint32_t* counts) {
    // cell -> [start,end) from the sorted keys of the point set
    std::vector<uint64_t> cells(size_t(np) + 1);
    std::vector<uint32_t> st(size_t(np) + 1), en(size_t(np) + 1);
    const int64_t m = orc_new_cell_ranges(np, psk, cells.data(), st.data(), en.data());
    auto find = [&](uint64_t key, uint32_t& s, uint32_t& e) {
        auto it = std::lower_bound(cells.begin(), cells.begin() + m, key);
        if (it == cells.begin() + m || *it != key) { s = e = 0; return; }
        const size_t k = size_t(it - cells.begin());
        s = st[k]; e = en[k];
    };
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nq; ++i) {
        const float* qi = q4 + 4 * i;
        const int cx = cell_coord(qi[0], g->origin[0], g->inv_cell, g->dims[0]);
        const int cy = cell_coord(qi[1], g->origin[1], g->inv_cell, g->dims[1]);
        const int cz = cell_coord(qi[2], g->origin[2], g->inv_cell, g->dims[2]);
        uint32_t c = 0;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = cx + dx, y = cy + dy, z = cz + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= g->dims[0] || y >= g->dims[1] || z >= g->dims[2]) continue;
                    const uint64_t key = new_key(g, x, y, z);
                    uint32_t s, e;
                    find(key, s, e);
                    for (uint32_t j = s; j < e; ++j) {
                        if (same_set && int64_t(j) == i) continue;
                        const float* pj = p4 + 4 * size_t(j);
                        const float ddx = qi[0] - pj[0], ddy = qi[1] - pj[1], ddz = qi[2] - pj[2];
                        const float d2 = std::fmaf(ddz, ddz, std::fmaf(ddy, ddy, ddx * ddx));
                        const float hij = 0.5f * (qi[3] + pj[3]);
                        if (d2 < hij * hij) c++;
                    }
                }
        counts[i] = c;
    }
}

}  // extern "C"
