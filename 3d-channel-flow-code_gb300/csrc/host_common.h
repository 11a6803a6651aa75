// Host-side helpers shared by the setup code and the synthetic-input
// generators: counter-based RNG and the sigma grid.
#pragma once
#include <cmath>
#include <cstdint>

#include "nsmp.h"

namespace nsmp {

// splitmix64 finaliser (Steele, Lea, Flood 2014).
inline uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Counter-based uniform in [0,1): a pure function of (seed, stream, index),
// so results do not depend on traversal order or renumbering.
inline double u01(uint64_t seed, uint64_t stream, uint64_t index) {
    uint64_t h = mix64(mix64(seed) ^ mix64(stream * 0xD1B54A32D192ED03ull + 1) ^ index);
    h = mix64(h ^ index);
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// Sigma grid (calcul_geometry.F90:263-283).  grid_kind 0 is the reference's
// uniform division; grid_kind 1 clusters levels toward both ends with
// z_j = a + (b-a)/2 (1 - tanh(beta(1-2j/L))/tanh(beta)), j = 0..L, L = NZ-2.
// Arrays are 0-based: sig[k-1] holds the reference's sig(k).
inline void sigma_grid(const nsmp_params& p, double* sig, double* dsig, double* sigv, double* dsigv) {
    const int NZ = p.nz;
    if (p.grid_kind == 0) {
        dsigv[0] = (p.sigfin - p.sigini) / (double)(float)(NZ - 2);
        sigv[0] = p.sigini;
        for (int k = 2; k <= NZ - 2; ++k) {
            dsigv[k - 1] = dsigv[0];
            sigv[k - 1] = sigv[k - 2] + dsigv[k - 2];
        }
        dsigv[NZ - 2] = dsigv[0];
        sigv[NZ - 2] = p.sigfin;
    } else {
        const int L = NZ - 2;
        const double tb = std::tanh(p.grid_beta);
        for (int j = 0; j <= L; ++j)
            sigv[j] = p.sigini + 0.5 * (p.sigfin - p.sigini) *
                                     (1.0 - std::tanh(p.grid_beta * (1.0 - 2.0 * j / L)) / tb);
        sigv[0] = p.sigini;
        sigv[NZ - 2] = p.sigfin;
        for (int k = 0; k <= NZ - 3; ++k) dsigv[k] = sigv[k + 1] - sigv[k];
        dsigv[NZ - 2] = dsigv[NZ - 3];
    }
    dsig[0] = dsigv[0];
    sig[0] = sigv[0] - 0.5 * dsigv[0];
    for (int k = 1; k <= NZ - 2; ++k) {
        dsig[k] = 0.5 * (dsigv[k] + dsigv[k - 1]);
        sig[k] = sig[k - 1] + dsig[k - 1];
    }
    dsig[NZ - 1] = dsigv[NZ - 2];
    sig[NZ - 1] = sig[NZ - 2] + dsig[NZ - 2];
}

}  // namespace nsmp
