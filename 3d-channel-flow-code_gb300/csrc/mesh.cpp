// Synthetic inputs: the periodic jittered triangle mesh (in the reference's
// data.txt layout) and the seeded channel initial state.  Neither exists in
// the reference, which ships no input decks.
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "host_common.h"

extern "C" int nsmp_mesh_size(int nx, int ny, int* n0, int* nvert) {
    if (nx < 2 || ny < 2 || !n0 || !nvert) return NSMP_ERR_ARG;
    *n0 = 2 * nx * ny;
    *nvert = (nx + 1) * (ny + 1);
    return NSMP_OK;
}

// Vertices are numbered row by row (nv = 1 + ix + iy*(nx+1)); boundary
// vertices are not jittered and lie exactly on the box edges, so the
// reference's coordinate-based periodic pairing (calcul_geometry.F90:484-512,
// 951-969) finds them.  Triangles are counter-clockwise, two per quad in
// quad order.
extern "C" int nsmp_mesh_generate(int nx, int ny, double x0, double x1, double y0, double y1,
                                  double jitter, unsigned long long seed, int* No_vp, int* No_cp,
                                  int* nbe, int* nbev, double* xv, double* yv) {
    if (nx < 2 || ny < 2 || !(x1 > x0) || !(y1 > y0) || jitter < 0.0 || jitter > 0.3) return NSMP_ERR_ARG;
    if (!No_vp || !No_cp || !nbe || !nbev || !xv || !yv) return NSMP_ERR_ARG;
    const int NV = (nx + 1) * (ny + 1), N0 = 2 * nx * ny;
    const double dx = (x1 - x0) / nx, dy = (y1 - y0) / ny;
    for (int iy = 0; iy <= ny; ++iy)
        for (int ix = 0; ix <= nx; ++ix) {
            int v = ix + iy * (nx + 1);
            bool bd = (ix == 0 || ix == nx || iy == 0 || iy == ny);
            double x = (ix == nx) ? x1 : x0 + ix * dx;
            double y = (iy == ny) ? y1 : y0 + iy * dy;
            if (!bd) {
                x += jitter * dx * (2.0 * nsmp::u01(seed, 1, 2ull * v) - 1.0);
                y += jitter * dy * (2.0 * nsmp::u01(seed, 1, 2ull * v + 1) - 1.0);
            }
            xv[v] = x;
            yv[v] = y;
            nbev[v] = bd ? 1 : 0;
        }
    auto vid = [&](int ix, int iy) { return 1 + ix + iy * (nx + 1); };
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
            int q = ix + iy * nx;
            int a = vid(ix, iy), b = vid(ix + 1, iy), c = vid(ix + 1, iy + 1), d = vid(ix, iy + 1);
            int t0 = 2 * q, t1 = 2 * q + 1;
            int tri[2][3];
            if (nsmp::u01(seed, 2, (uint64_t)q) < 0.5) {  // diagonal a-c
                int A[3] = {a, b, c}, B[3] = {a, c, d};
                std::memcpy(tri[0], A, sizeof A); std::memcpy(tri[1], B, sizeof B);
            } else {                                       // diagonal b-d
                int A[3] = {a, b, d}, B[3] = {b, c, d};
                std::memcpy(tri[0], A, sizeof A); std::memcpy(tri[1], B, sizeof B);
            }
            for (int j = 0; j < 3; ++j) {
                No_vp[t0 + j * N0] = tri[0][j];
                No_vp[t1 + j * N0] = tri[1][j];
            }
        }
    // Neighbour across edge j (v_j -> v_{j+1}); 0 on the boundary.
    std::map<std::pair<int, int>, int> edge;
    for (int t = 0; t < N0; ++t)
        for (int j = 0; j < 3; ++j) {
            int va = No_vp[t + j * N0], vb = No_vp[t + ((j + 1) % 3) * N0];
            edge[{va, vb}] = t + 1;
        }
    for (int t = 0; t < N0; ++t) {
        nbe[t] = 0;
        for (int j = 0; j < 3; ++j) {
            int va = No_vp[t + j * N0], vb = No_vp[t + ((j + 1) % 3) * N0];
            auto it = edge.find({vb, va});
            No_cp[t + j * N0] = (it == edge.end()) ? 0 : it->second;
            if (it == edge.end()) nbe[t] = 1;
        }
    }
    // Positive orientation check (areas must be > 0 after jitter).
    for (int t = 0; t < N0; ++t) {
        int v1 = No_vp[t] - 1, v2 = No_vp[t + N0] - 1, v3 = No_vp[t + 2 * N0] - 1;
        double ar = (xv[v2] - xv[v1]) * (yv[v3] - yv[v1]) - (xv[v3] - xv[v1]) * (yv[v2] - yv[v1]);
        if (!(ar > 0.0)) return NSMP_ERR_MESH;
    }
    (void)NV;
    return NSMP_OK;
}

extern "C" int nsmp_sigma_grid(const nsmp_params* prm, double* sig, double* dsig, double* sigv, double* dsigv) {
    if (!prm || prm->nz < 4 || !sig || !dsig || !sigv || !dsigv) return NSMP_ERR_ARG;
    nsmp::sigma_grid(*prm, sig, dsig, sigv, dsigv);
    return NSMP_OK;
}

// Channel initial state: the reference's profile umax*z*(2-z)
// (Functions.F90:22-31) with uniform noise.  The reference's noise comes from
// random_seed/random_number with an unseeded generator (Functions.F90:26-27),
// so a counter-based generator keyed by the original cell number replaces it.
extern "C" int nsmp_initial_channel(const nsmp_params* prm, int n_cell, double umax, double amp,
                                    unsigned long long seed, double* u, double* v, double* w, double* p) {
    if (!prm || n_cell < prm->n0 || !u || !v || !w || !p) return NSMP_ERR_ARG;
    const int NZ = prm->nz, N0 = prm->n0;
    std::vector<double> sig(NZ), dsig(NZ), sigv(NZ - 1), dsigv(NZ - 1);
    nsmp::sigma_grid(*prm, sig.data(), dsig.data(), sigv.data(), dsigv.data());
    for (int k = 0; k < NZ; ++k)
        for (int i = 0; i < n_cell; ++i) {
            size_t q = (size_t)i + (size_t)k * n_cell;
            u[q] = v[q] = w[q] = p[q] = 0.0;
            double z = sig[k];
            if (i >= N0 || z < prm->sigini || z > prm->sigfin) continue;
            uint64_t key = ((uint64_t)(i + 1) << 20) ^ (uint64_t)(k + 1);
            u[q] = umax * z * (2.0 - z) + amp * (2.0 * nsmp::u01(seed, 11, key) - 1.0);
            v[q] = amp * (2.0 * nsmp::u01(seed, 12, key) - 1.0);
            w[q] = amp * (2.0 * nsmp::u01(seed, 13, key) - 1.0);
        }
    return NSMP_OK;
}
