// Seeded random sequential insertion of non-overlapping spheres (scene generation).
//
// Host-side helper used to build the synthetic scenes of the benchmark and the tests; it
// plays the role of SpherePack::makeCloud (lib/sphere-pack/SpherePack.hpp:75) for the region
// shapes those scenes need. Spheres are inserted in the given order (largest first packs
// densest); each gets up to max_attempts uniformly drawn candidate centres and is accepted
// at the first one that overlaps no previously placed sphere.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace {

struct Rng {  // splitmix64 -> uniform doubles
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace

extern "C" {

/* region_kind 0: box lo..hi (spheres fully inside).
   region_kind 1: cylinder with axis x through (params[0], params[1]) = (y0, z0), radius params[2],
                  x in [lo.x, hi.x], keeping only z <= params[3]; spheres fully inside.
   region_kind 2: periodic box lo..hi (distances wrap on all axes).
   Returns the number of placed spheres (== n on success). */
int64_t wg_pack_rsa(int64_t n, const double* radii, const double* lo, const double* hi, int32_t region_kind,
                    const double* params, uint64_t seed, int64_t max_attempts, double* centers) {
    if (n <= 0) return 0;
    double rmax = 0;
    for (int64_t i = 0; i < n; i++) rmax = std::fmax(rmax, radii[i]);
    const double cs = 2 * rmax;
    const double L[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    int64_t nc[3];
    for (int k = 0; k < 3; k++) nc[k] = std::max<int64_t>(1, (int64_t)std::floor(L[k] / cs));
    const double cw[3] = {L[0] / nc[0], L[1] / nc[1], L[2] / nc[2]};
    std::vector<std::vector<int32_t>> cells((size_t)(nc[0] * nc[1] * nc[2]));
    Rng rng{seed * 0x2545F4914F6CDD1Dull + 12345};
    const bool peri = (region_kind == 2);
    int64_t placed = 0;
    for (int64_t i = 0; i < n; i++) {
        const double r = radii[i];
        bool ok = false;
        for (int64_t a = 0; a < max_attempts && !ok; a++) {
            double c[3];
            for (int k = 0; k < 3; k++) {
                double m = peri ? 0 : r;
                c[k] = lo[k] + m + rng.uni() * (L[k] - 2 * m);
            }
            if (region_kind == 1) {
                double dy = c[1] - params[0], dz = c[2] - params[1];
                if (std::sqrt(dy * dy + dz * dz) > params[2] - r) continue;
                if (c[2] + r > params[3]) continue;
            }
            int64_t ci[3];
            for (int k = 0; k < 3; k++) {
                ci[k] = (int64_t)std::floor((c[k] - lo[k]) / cw[k]);
                if (ci[k] < 0) ci[k] = 0;
                if (ci[k] >= nc[k]) ci[k] = nc[k] - 1;
            }
            bool clash = false;
            for (int dz = -1; dz <= 1 && !clash; dz++)
                for (int dy = -1; dy <= 1 && !clash; dy++)
                    for (int dx = -1; dx <= 1 && !clash; dx++) {
                        int64_t q[3] = {ci[0] + dx, ci[1] + dy, ci[2] + dz};
                        bool skip = false;
                        for (int k = 0; k < 3; k++) {
                            if (q[k] < 0 || q[k] >= nc[k]) {
                                if (!peri) skip = true;
                                else q[k] = (q[k] + nc[k]) % nc[k];
                            }
                        }
                        if (skip) continue;
                        for (int32_t j : cells[(size_t)((q[2] * nc[1] + q[1]) * nc[0] + q[0])]) {
                            double d2 = 0;
                            for (int k = 0; k < 3; k++) {
                                double d = c[k] - centers[3 * j + k];
                                if (peri) d -= L[k] * std::round(d / L[k]);
                                d2 += d * d;
                            }
                            double rr = r + radii[j];
                            if (d2 < rr * rr) { clash = true; break; }
                        }
                    }
            if (clash) continue;
            for (int k = 0; k < 3; k++) centers[3 * i + k] = c[k];
            cells[(size_t)((ci[2] * nc[1] + ci[1]) * nc[0] + ci[0])].push_back((int32_t)i);
            ok = true;
        }
        if (!ok) return placed;
        placed++;
    }
    return placed;
}
}
