// Host setup: geometry of the prismatic sigma grid and the device tables.
//
// Restates what the Fortran driver computes once before the time loop --
// calcul_geometry (Main/calcul_geometry.F90:263-1517, serial branches),
// adjust_tagv/adjust_bc (BoundaryConditions/update_bc.F90:4-513) and the
// coefficients of PDE_center (AdvectionDiffusion/PDE.F90:69-121) -- with the
// reference's arithmetic, then turns the result into the column-major device
// layout described in layout.h.  The O(N^2) searches of the reference
// (periodic vertex pairing, vertex stencils) are replaced by coordinate and
// edge maps that visit the same candidates and give the same results.
#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <map>
#include <numeric>
#include <queue>
#include <tuple>

#include "host_common.h"
#include "layout.h"
#include "setup_geo.h"

namespace nsmp {
namespace setup {
namespace {

const double kTolF = (double)1.0E-7f;  // default-REAL literal 1.0E-7 of the reference
const double kTolD = 1.0e-7;           // 1.0d-7

// Quantised coordinate key with a +-1 neighbourhood lookup, verified with the
// reference's tolerance; equivalent to scanning every boundary vertex.
struct CoordIndex {
    std::map<std::pair<long long, long long>, std::vector<int>> m;
    static long long q(double x) { return (long long)std::llround(x * 1.0e6); }
    void add(double x, double y, int id) { m[{q(x), q(y)}].push_back(id); }
    template <class F>
    void each_near(double x, double y, F f) const {
        long long qx = q(x), qy = q(y);
        for (long long a = qx - 1; a <= qx + 1; ++a)
            for (long long b = qy - 1; b <= qy + 1; ++b) {
                auto it = m.find({a, b});
                if (it == m.end()) continue;
                for (int id : it->second) f(id);
            }
    }
};

}  // namespace

// Cell centres, areas, edges, normals: calcul_geometry.F90:292-367.  The
// centre and area arrays leave room for one ghost cell per boundary edge.
void cell_geometry(Geo& g) {
    const int N0 = g.N0;
    int nghost = 0;
    for (int i = 0; i < N0; ++i)
        for (int j = 0; j < 3; ++j)
            if (g.cp[g.at(i, j)] < 0) ++nghost;
    const int NCmax = N0 + nghost;
    g.xc.assign(NCmax, 0.0); g.yc.assign(NCmax, 0.0); g.area.assign(NCmax, 0.0);
    for (auto* a : {&g.dxVV, &g.dyVV, &g.dlVV, &g.xnn, &g.ynn}) a->assign(3 * N0, 0.0);
    double vol = 0.0;
    for (int i = 0; i < N0; ++i) {
        const int v1 = g.vp[g.at(i, 0)], v2 = g.vp[g.at(i, 1)], v3 = g.vp[g.at(i, 2)];
        g.xc[i] = (g.xv[v1] + g.xv[v2] + g.xv[v3]) / 3.0;
        g.yc[i] = (g.yv[v1] + g.yv[v2] + g.yv[v3]) / 3.0;
        g.area[i] = 0.5 * std::fabs(g.xv[v1] * (g.yv[v2] - g.yv[v3]) + g.xv[v2] * (g.yv[v3] - g.yv[v1]) +
                                    g.xv[v3] * (g.yv[v1] - g.yv[v2]));
        const int vv[4] = {v1, v2, v3, v1};
        for (int j = 0; j < 3; ++j) {
            g.dxVV[g.at(i, j)] = g.xv[vv[j + 1]] - g.xv[vv[j]];
            g.dyVV[g.at(i, j)] = g.yv[vv[j + 1]] - g.yv[vv[j]];
        }
        for (int j = 0; j < 3; ++j) {
            const int q = g.at(i, j);
            g.dlVV[q] = std::sqrt(g.dxVV[q] * g.dxVV[q] + g.dyVV[q] * g.dyVV[q]);
        }
        for (int j = 0; j < 3; ++j) {
            const int q = g.at(i, j);
            g.xnn[q] = g.dyVV[q] / g.dlVV[q];
            g.ynn[q] = -g.dxVV[q] / g.dlVV[q];
        }
        vol = vol + g.area[i];
    }
    g.total_volume = vol;
}

// Ghost cells with their periodic images (calcul_geometry.F90:402-578) and
// the periodic vertex pairs and corners (:893-1040).
int ghosts_and_pairs(const nsmp_params& p, Geo& g, std::string& err) {
    const int N0 = g.N0, NV = g.NV;
    int nghost = 0;
    for (int i = 0; i < N0; ++i)
        for (int j = 0; j < 3; ++j)
            if (g.cp[g.at(i, j)] < 0) ++nghost;
    const int NCmax = N0 + nghost;
    // boundary vertex coordinate index and boundary edge -> cell map
    CoordIndex bidx;
    for (int nv = 0; nv < NV; ++nv)
        if (g.nbev[nv] != 0) bidx.add(g.xv[nv], g.yv[nv], nv);
    std::map<std::pair<int, int>, std::vector<int>> bedge;  // undirected edge -> boundary cells
    for (int i = 0; i < N0; ++i) {
        if (g.nbe[i] == 0) continue;
        for (int j = 0; j < 3; ++j) {
            int a = g.vp[g.at(i, j)], b = g.vp[g.at(i, (j + 1) % 3)];
            bedge[{std::min(a, b), std::max(a, b)}].push_back(i);
        }
    }

    // ghost cells and periodic images: calcul_geometry.F90:402-578
    const double Lx = p.xdfin - p.xdini, Ly = p.ydfin - p.ydini;
    g.cp.resize(3 * (size_t)NCmax, -1);
    // cp is (N0,3) column-major; rebuild with the larger leading dimension.
    {
        std::vector<int> cp2(3 * (size_t)NCmax, -1);
        for (int i = 0; i < N0; ++i)
            for (int j = 0; j < 3; ++j) cp2[i + (size_t)j * NCmax] = g.cp[i + (size_t)j * N0];
        g.cp.swap(cp2);
    }
    auto CP = [&](int i, int j) -> int& { return g.cp[i + (size_t)j * NCmax]; };
    g.img.clear();
    int ii = N0;
    for (int i = 0; i < N0; ++i) {
        if (g.nbe[i] <= 0) continue;
        for (int j = 0; j < 3; ++j) {
            if (CP(i, j) >= 0) continue;
            const int gh = ii++;
            CP(i, j) = gh;
            g.area[gh] = g.area[i];
            const int jv1 = g.vp[g.at(i, j)], jv2 = g.vp[g.at(i, (j + 1) % 3)];
            const double dx = g.dxVV[g.at(i, j)], dy = g.dyVV[g.at(i, j)];
            double xee, yee;
            if (std::fabs(dy) < kTolF) {
                yee = g.yv[jv2];
                xee = g.xc[i];
            } else {
                const double r = dx / dy, r2 = r * r;
                yee = (g.yc[i] - (g.xv[jv2] - g.xc[i]) * r + g.yv[jv2] * r2) / (1.0 + r2);
                xee = g.xv[jv2] + (yee - g.yv[jv2]) * r;
            }
            const double xm = 2.0 * xee - g.xc[i], ym = 2.0 * yee - g.yc[i];
            double sx = Lx, sy = Ly;
            if (xm > p.xdfin) { sx = -1.0 * sx; sy = 0.0; } else if (xm < p.xdini) { sy = 0.0; }
            if (ym > p.ydfin) { sx = 0.0; sy = -1.0 * sy; } else if (ym < p.ydini) { sx = 0.0; }
            if (sx * sy > kTolF) {
                err = "ghost cell without periodic image: only periodic lateral boundaries are supported";
                return NSMP_ERR_UNSUPPORTED;
            }
            auto find_vertex = [&](double x, double y) {
                int found = -1, n = 0;
                bidx.each_near(x, y, [&](int nv) {
                    if (std::fabs(x - g.xv[nv]) < kTolF && std::fabs(y - g.yv[nv]) < kTolF) { found = nv; ++n; }
                });
                return n == 1 ? found : -1;
            };
            const int p1 = find_vertex(g.xv[jv1] + sx, g.yv[jv1] + sy);
            const int p2 = find_vertex(g.xv[jv2] + sx, g.yv[jv2] + sy);
            if (p1 < 0 || p2 < 0) { err = "periodic vertex pair not found"; return NSMP_ERR_MESH; }
            auto it = bedge.find({std::min(p1, p2), std::max(p1, p2)});
            if (it == bedge.end() || it->second.size() != 1) { err = "periodic image cell not found"; return NSMP_ERR_MESH; }
            const int im = it->second[0];
            int cc = -1;
            for (int q = 0; q < 3; ++q) {
                int v = g.vp[g.at(im, q)];
                if (v != p1 && v != p2) cc = v;
            }
            g.xc[gh] = (g.xv[jv1] + g.xv[jv2] + (g.xv[cc] - sx)) / 3.0;
            g.yc[gh] = (g.yv[jv1] + g.yv[jv2] + (g.yv[cc] - sy)) / 3.0;
            g.img.push_back(im);
        }
    }
    g.NC = ii;

    // vertex tags, corners and periodic pairs: calcul_geometry.F90:893-1040
    g.vpair.assign(NV, -1); g.vedge.assign(NV, -1);
    std::vector<int> tx(NV, 0), ty(NV, 0);
    for (int nv = 0; nv < NV; ++nv) {
        if (g.nbev[nv] == 0) continue;
        if (std::fabs(g.xv[nv] - p.xdini) < kTolD) tx[nv] = 1;
        if (std::fabs(g.xv[nv] - p.xdfin) < kTolD) tx[nv] = 2;
        if (std::fabs(g.yv[nv] - p.ydini) < kTolD) ty[nv] = 1;
        if (std::fabs(g.yv[nv] - p.ydfin) < kTolD) ty[nv] = 2;
    }
    int ncorner = 0;
    for (int nv = 0; nv < NV; ++nv) {
        if (tx[nv] * ty[nv] > 0) { g.vedge[nv] = 1; ++ncorner; continue; }
        if (tx[nv] == 0 && ty[nv] == 0) continue;
        // partner across the box; the reference accepts any boundary vertex
        // at the same abscissa (ordinate) and box-length distance
        int n = 0, pr = -1;
        const double cand[2][2] = {{g.xv[nv], ty[nv] == 1 ? p.ydfin : p.ydini},
                                   {tx[nv] == 1 ? p.xdfin : p.xdini, g.yv[nv]}};
        const int which = (ty[nv] > 0) ? 0 : 1;
        bidx.each_near(cand[which][0], cand[which][1], [&](int i) {
            bool ymatch = std::fabs(g.xv[nv] - g.xv[i]) < kTolD && std::fabs(g.yv[nv] - g.yv[i]) > (Ly - kTolD);
            bool xmatch = std::fabs(g.yv[nv] - g.yv[i]) < kTolD && std::fabs(g.xv[nv] - g.xv[i]) > (Lx - kTolD);
            if (ymatch || xmatch) { ++n; pr = i; }
        });
        if (n != 1) { err = "missing periodic partner of a boundary vertex"; return NSMP_ERR_MESH; }
        g.vpair[nv] = pr;
    }
    if (ncorner != 4) { err = "expected 4 corner vertices"; return NSMP_ERR_MESH; }
    return 0;
}

// The cells around each vertex in the reference's visiting order (cell, then
// corner): CSR over vertices of 3 * cell + corner.
void vertex_incidence(const Geo& g, std::vector<int>& ptr, std::vector<int>& inc) {
    ptr.assign(g.NV + 1, 0);
    for (int i = 0; i < g.N0; ++i)
        for (int j = 0; j < 3; ++j) ptr[g.vp[g.at(i, j)] + 1] += 1;
    for (int v = 0; v < g.NV; ++v) ptr[v + 1] += ptr[v];
    inc.assign(3 * (size_t)g.N0, 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < g.N0; ++i)
        for (int j = 0; j < 3; ++j) inc[fill[g.vp[g.at(i, j)]]++] = 3 * i + j;
}

// Vertex stencils (surrounding/weight/dlVsum): calcul_geometry.F90:1055-1076.
void vertex_weights(Geo& g) {
    const int N0 = g.N0, NV = g.NV;
    g.stencil.assign(NV, {});
    g.dlVsum.assign(NV, 0.0);
    for (int i = 0; i < N0; ++i)
        for (int j = 0; j < 3; ++j) {
            const int nv = g.vp[g.at(i, j)];
            const double dx = g.xc[i] - g.xv[nv], dy = g.yc[i] - g.yv[nv];
            const double w = 1.0 / std::sqrt(dx * dx + dy * dy);
            g.stencil[nv].push_back({i, w});
            g.dlVsum[nv] = g.dlVsum[nv] + w;
        }
}

// Edge midpoints, centre-line intersections, doe (calcul_geometry.F90:1343-1387);
// LSQ sums and Kim-Choi factors (:1460-1517).
void edge_geometry(Geo& g) {
    const int N0 = g.N0;
    const size_t NCmax = g.cp.size() / 3;
    auto CP = [&](int i, int j) { return g.cp[i + (size_t)j * NCmax]; };
    g.doe.assign(3 * N0, 0.0);
    for (int i = 0; i < N0; ++i)
        for (int j = 0; j < 3; ++j) {
            const int jv1 = g.vp[g.at(i, j)], jv2 = g.vp[g.at(i, (j + 1) % 3)], jc = CP(i, j);
            const double xme = 0.5 * (g.xv[jv2] + g.xv[jv1]), yme = 0.5 * (g.yv[jv2] + g.yv[jv1]);
            const double x1 = g.xc[i], x2 = g.xc[jc], x3 = g.xv[jv1], x4 = g.xv[jv2];
            const double y1 = g.yc[i], y2 = g.yc[jc], y3 = g.yv[jv1], y4 = g.yv[jv2];
            const double den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
            const double xmo = ((x1 * y2 - y1 * x2) * (x3 - x4) - (x1 - x2) * (x3 * y4 - y3 * x4)) / den;
            const double ymo = ((x1 * y2 - y1 * x2) * (y3 - y4) - (y1 - y2) * (x3 * y4 - y3 * x4)) / den;
            const double ex = xme - xmo, ey = yme - ymo;
            double d = std::sqrt(ex * ex + ey * ey);
            if (ex * g.dxVV[g.at(i, j)] + ey * g.dyVV[g.at(i, j)] < 0.0) d = -d;
            g.doe[g.at(i, j)] = d;
        }

    // LSQ sums and Kim-Choi factors: calcul_geometry.F90:1460-1517
    for (auto* a : {&g.dxCC, &g.dyCC, &g.dlCC, &g.dle1, &g.dle2}) a->assign(3 * N0, 0.0);
    g.sxx.assign(N0, 0.0); g.syy.assign(N0, 0.0); g.sxy.assign(N0, 0.0);
    for (int i = 0; i < N0; ++i) {
        double sX = 0.0, sY = 0.0, sXY = 0.0;
        for (int j = 0; j < 3; ++j) {
            const int q = g.at(i, j), jc = CP(i, j);
            const double dx = g.xc[jc] - g.xc[i], dy = g.yc[jc] - g.yc[i];
            const double dl = std::sqrt(dx * dx + dy * dy);
            g.dxCC[q] = dx; g.dyCC[q] = dy; g.dlCC[q] = dl;
            sX = sX + dx * dx;
            sY = sY + dy * dy;
            sXY = sXY + dx * dy;
            double ux = dx / dl, uy = dy / dl;
            double cth = ux * g.xnn[q] + uy * g.ynn[q];
            ux = ux / cth;
            uy = uy / cth;
            g.dle1[q] = 1.0 / cth;
            const double tx2 = g.xnn[q] - ux, ty2 = g.ynn[q] - uy;
            const double s = tx2 * g.dxVV[q] + ty2 * g.dyVV[q];
            g.dle2[q] = (s < 0.0) ? -1.0 * std::sqrt(tx2 * tx2 + ty2 * ty2) : std::sqrt(tx2 * tx2 + ty2 * ty2);
        }
        g.sxx[i] = sX; g.syy[i] = sY; g.sxy[i] = sXY;
    }
}

namespace {

// Reverse Cuthill-McKee over the periodic triangle adjacency; ties broken by
// (degree, original number) so the permutation is deterministic.
std::vector<int> rcm(int N0, const std::vector<std::array<int, 3>>& adj) {
    std::vector<int> order;
    order.reserve(N0);
    std::vector<char> seen(N0, 0);
    auto deg = [&](int c) {
        int d = 0;
        for (int q = 0; q < 3; ++q) if (adj[c][q] >= 0 && adj[c][q] != c) ++d;
        return d;
    };
    for (int s0 = 0; s0 < N0; ++s0) {
        if (seen[s0]) continue;
        // every cell of a periodic triangulation has degree 3: start each
        // component at its lowest original number
        int start = s0;
        std::queue<int> q;
        q.push(start);
        seen[start] = 1;
        while (!q.empty()) {
            int c = q.front();
            q.pop();
            order.push_back(c);
            std::array<int, 3> nb = adj[c];
            std::sort(nb.begin(), nb.end(), [&](int a, int b) {
                if (a < 0 || b < 0) return a > b;
                return std::make_pair(deg(a), a) < std::make_pair(deg(b), b);
            });
            for (int n : nb)
                if (n >= 0 && !seen[n]) { seen[n] = 1; q.push(n); }
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

}  // namespace

int read_mesh(const nsmp_params& p, const nsmp_mesh& m, Geo& g, std::string& err) {
    if (p.n0 <= 0 || p.nvert <= 0 || p.nz < 4) { err = "bad sizes"; return NSMP_ERR_ARG; }
    if (!(p.xdfin > p.xdini) || !(p.ydfin > p.ydini) || !(p.sigfin > p.sigini)) { err = "bad box"; return NSMP_ERR_ARG; }
    if (p.top_bc < 0 || p.top_bc > 1 || p.bot_bc < 0 || p.bot_bc > 1) {
        err = "TopBC/BotBC must be 0 (no-slip) or 1 (free-slip)";
        return NSMP_ERR_UNSUPPORTED;
    }
    if (!(p.dt > 0.0) || !(p.re > 0.0) || !(p.eps > 0.0) || p.max_iters < 0) { err = "bad dt/Re/eps/MaxIters"; return NSMP_ERR_ARG; }
    g.N0 = p.n0; g.NV = p.nvert; g.NZ = p.nz;
    g.vp.resize(3 * (size_t)g.N0); g.cp.resize(3 * (size_t)g.N0);
    g.nbe.assign(m.nbe, m.nbe + g.N0); g.nbev.assign(m.nbev, m.nbev + g.NV);
    g.xv.assign(m.xv, m.xv + g.NV); g.yv.assign(m.yv, m.yv + g.NV);
    for (size_t q = 0; q < 3 * (size_t)g.N0; ++q) {
        if (m.No_vp[q] < 1 || m.No_vp[q] > g.NV || m.No_cp[q] < 0 || m.No_cp[q] > g.N0) {
            err = "mesh index out of range";
            return NSMP_ERR_MESH;
        }
        g.vp[q] = m.No_vp[q] - 1;
        g.cp[q] = m.No_cp[q] - 1;
    }
    return 0;
}

// Adjacency, renumbering, vertex classes and stencils, the sigma grid and
// level factors, and the device tables in the new column order, from the
// finished geometry.
int finish_layout(const nsmp_params& p, Geo& g, HostLayout& L, std::string& err) {
    const int N0 = g.N0, NV = g.NV, NZ = g.NZ, NC = g.NC;
    const size_t NCmax = g.cp.size() / 3;
    auto CP = [&](int i, int j) { return g.cp[i + (size_t)j * NCmax]; };

    L.N0 = N0; L.NV = NV; L.NZ = NZ; L.NZI = NZ - 2; L.NC = NC;
    L.total_volume = g.total_volume;
    L.lsig = p.sigfin - p.sigini;
    L.ghost_img = g.img;

    // periodic adjacency of interior cells
    std::vector<std::array<int, 3>> adj(N0);
    for (int i = 0; i < N0; ++i)
        for (int j = 0; j < 3; ++j) {
            int c = CP(i, j);
            adj[i][j] = (c < N0) ? c : g.img[c - N0];
        }
    L.perm = rcm(N0, adj);
    if ((int)L.perm.size() != N0) { err = "renumbering failed"; return NSMP_ERR_MESH; }
    L.iperm.assign(N0, -1);
    for (int c = 0; c < N0; ++c) L.iperm[L.perm[c]] = c;

    // periodic vertex classes (bc_periodic, BC.F90:1243-1300): pairs and the
    // four corners share one value.
    std::vector<int> rep(NV);
    std::iota(rep.begin(), rep.end(), 0);
    std::function<int(int)> find = [&](int a) { return rep[a] == a ? a : rep[a] = find(rep[a]); };
    auto unite = [&](int a, int b) { a = find(a); b = find(b); if (a != b) rep[std::max(a, b)] = std::min(a, b); };
    std::vector<int> corners;
    for (int nv = 0; nv < NV; ++nv) {
        if (g.vedge[nv] == 1) corners.push_back(nv);
        else if (g.vpair[nv] >= 0) unite(nv, g.vpair[nv]);
    }
    for (size_t q = 1; q < corners.size(); ++q) unite(corners[0], corners[q]);
    // class numbers in order of first use by the renumbered columns
    L.vclass.assign(NV, -1);
    std::vector<int> root_class(NV, -1);
    int ncls = 0;
    for (int c = 0; c < N0; ++c) {
        int i = L.perm[c];
        for (int j = 0; j < 3; ++j) {
            int r = find(g.vp[g.at(i, j)]);
            if (root_class[r] < 0) root_class[r] = ncls++;
        }
    }
    for (int nv = 0; nv < NV; ++nv) {
        int r = find(nv);
        if (root_class[r] < 0) root_class[r] = ncls++;  // vertex without cells (not in a valid mesh)
        L.vclass[nv] = root_class[r];
    }
    L.nclass = ncls;
    // merged stencil: coefficient w / (sum of dlVsum over the class members);
    // members in ascending vertex number, cells in the reference's order.
    std::vector<std::vector<int>> members(ncls);
    for (int nv = 0; nv < NV; ++nv) members[L.vclass[nv]].push_back(nv);
    L.vptr.assign(ncls + 1, 0);
    L.vcell.clear(); L.vcoef.clear();
    for (int v = 0; v < ncls; ++v) {
        double S = 0.0;
        if (members[v].size() == 4) {  // corners: summed in corner-list order
            for (int nv : corners) S = S + g.dlVsum[nv];
        } else if (members[v].size() == 2) {
            S = g.dlVsum[members[v][0]] + g.dlVsum[members[v][1]];
        } else {
            S = g.dlVsum[members[v][0]];
        }
        for (int nv : members[v])
            for (auto& cw : g.stencil[nv]) {
                L.vcell.push_back(L.iperm[cw.first]);
                L.vcoef.push_back(cw.second / S);
            }
        L.vptr[v + 1] = (int)L.vcell.size();
    }

    // sigma grid and per-layer factors
    L.sig.resize(NZ); L.dsig.resize(NZ); L.sigv.resize(NZ - 1); L.dsigv.resize(NZ - 1);
    sigma_grid(p, L.sig.data(), L.dsig.data(), L.sigv.data(), L.dsigv.data());
    Levels& lv = L.lev;
    for (auto* a : {&lv.dsv, &lv.idsT, &lv.idsB, &lv.idsBu, &lv.wT, &lv.wB, &lv.gzp, &lv.gzm, &lv.hmean,
                    &lv.les_dd, &lv.les_kd, &lv.les_damp, &lv.ihz, &lv.cfl_div, &lv.cfl_h})
        a->assign(NZ, 0.0);
    const bool compat = p.ref_bug_compat != 0;
    const double von_karman = (double)0.415f;  // module_les.F90:33, a REAL literal
    for (int k0 = 1; k0 <= NZ - 2; ++k0) {
        // reference layer k = k0+1; sig(k) = L.sig[k0], dsigv(k-1) = L.dsigv[k0-1]
        lv.dsv[k0] = L.dsigv[k0 - 1];
        lv.idsT[k0] = 1.0 / L.dsig[k0];
        lv.idsB[k0] = 1.0 / L.dsig[k0 - 1];
        lv.idsBu[k0] = compat ? 1.0 / L.dsig[k0] : 1.0 / L.dsig[k0 - 1];
        lv.wT[k0] = (k0 == NZ - 2) ? 0.0 : 1.0;
        lv.wB[k0] = (k0 == 1) ? 0.0 : 1.0;
        const double dzp = L.sig[k0 + 1] - L.sig[k0], dzm = L.sig[k0 - 1] - L.sig[k0];
        const double ss = dzp * dzp + dzm * dzm;
        lv.gzp[k0] = dzp / ss;
        lv.gzm[k0] = dzm / ss;
        lv.hmean[k0] = compat ? L.dsig[k0] : L.dsigv[k0 - 1];
        const double z = L.sig[k0];
        double wd = std::fabs(z);
        if (!compat) {
            wd = std::fabs(z - p.sigini);
            if (p.top_bc == 0) wd = std::min(wd, std::fabs(p.sigfin - z));
        }
        lv.les_dd[k0] = 0.1 * std::cbrt(L.dsig[k0]);
        lv.les_kd[k0] = von_karman * wd;
        lv.les_damp[k0] = 1.0 - std::exp(-(wd * 1.0 * p.re) / 26.0);
        lv.ihz[k0] = compat ? 1.0 / L.dsig[k0] : 1.0 / L.dsigv[k0 - 1];
        // glob_cfl weights its lateral fluxes by dsig(k-1) in the divergence
        // and by dsig(k) in the CFL number, side flux and volume means
        // (cfl.F90:108-110, 139-140, 151, 161); the cell height is dsigv(k-1)
        lv.cfl_div[k0] = compat ? L.dsig[k0 - 1] : L.dsigv[k0 - 1];
        lv.cfl_h[k0] = compat ? L.dsig[k0] : L.dsigv[k0 - 1];
    }
    for (int c = 0; c < 3; ++c) {
        L.sgn_bot[c] = (p.bot_bc == 0 || c == 2) ? -1.0 : 1.0;
        L.sgn_top[c] = (p.top_bc == 0 || c == 2) ? -1.0 : 1.0;
    }

    // per-column tables in the new order
    L.ppe.resize(N0);
    L.geo.resize(N0);
    for (int c = 0; c < N0; ++c) {
        const int i = L.perm[c];
        ColPPE& P = L.ppe[c];
        ColGeo& G = L.geo[c];
        const double sxx = g.sxx[i], syy = g.syy[i], sxy = g.sxy[i];
        const double det = sxx * syy - sxy * sxy;
        P.pad = 0;
        G.bnd = 0;
        G.orig = i;
        for (int j = 0; j < 3; ++j) {
            const int q = g.at(i, j);
            const int nbc = L.iperm[adj[i][j]];
            P.nb[j] = nbc;
            G.nb[j] = nbc;
            if (CP(i, j) >= N0) G.bnd |= 1 << j;
            G.vtx[j] = L.vclass[g.vp[q]];
            const double co1 = g.dle1[q] / g.dlCC[q];
            P.kA[j] = co1 * g.dlVV[q];
            G.kA[j] = P.kA[j];
            G.dle2[j] = g.dle2[q];
            G.cA[j] = co1;
            G.cB[j] = g.dle2[q] / g.dlVV[q];
            G.kE[j] = g.doe[q] / g.dlVV[q];
            G.L[j] = g.dlVV[q];
            G.xn[j] = g.xnn[q];
            G.yn[j] = g.ynn[q];
            G.gx[j] = (syy * g.dxCC[q] - sxy * g.dyCC[q]) / det;
            G.gy[j] = (sxx * g.dyCC[q] - sxy * g.dxCC[q]) / det;
            G.lxu[j] = g.xnn[q] * g.dlVV[q] / g.area[i];
            G.lyu[j] = g.ynn[q] * g.dlVV[q] / g.area[i];
            // sgm_les.F90:445-446, 454-455: v pairs face 2 with dlVV(i,3), face 3 with dlVV(i,2)
            const int jl = compat ? (j == 0 ? 0 : (j == 1 ? 2 : 1)) : j;
            G.lxv[j] = g.xnn[q] * g.dlVV[g.at(i, jl)] / g.area[i];
            G.lyv[j] = g.ynn[q] * g.dlVV[g.at(i, jl)] / g.area[i];
        }
        P.area = g.area[i];
        G.area = g.area[i];
        G.inv_area = 1.0 / g.area[i];
        G.cbrt_area = std::cbrt(g.area[i]);
    }

    // reference-shaped diagnostics
    L.ref_xc.assign(g.xc.begin(), g.xc.begin() + NC);
    L.ref_yc.assign(g.yc.begin(), g.yc.begin() + NC);
    L.ref_area.assign(g.area.begin(), g.area.begin() + NC);
    L.ref_dlVV = g.dlVV; L.ref_dlCC = g.dlCC; L.ref_dle1 = g.dle1; L.ref_dle2 = g.dle2;
    L.ref_doe = g.doe; L.ref_xnn = g.xnn; L.ref_ynn = g.ynn; L.ref_dxCC = g.dxCC; L.ref_dyCC = g.dyCC;
    L.ref_sxx = g.sxx; L.ref_syy = g.syy; L.ref_sxy = g.sxy;
    L.ref_dlVsum = g.dlVsum;
    L.ref_No_cp.assign(3 * (size_t)NC, 0);
    for (int i = 0; i < N0; ++i)
        for (int j = 0; j < 3; ++j) L.ref_No_cp[i + (size_t)j * NC] = CP(i, j) + 1;
    for (int gh = N0; gh < NC; ++gh) L.ref_No_cp[gh + 2 * (size_t)NC] = g.img[gh - N0] + 1;
    return 0;
}

}  // namespace setup

// The whole setup on the host: the reference's arithmetic step by step.
int build_layout(const nsmp_params& p, const nsmp_mesh& m, HostLayout& L, std::string& err) {
    setup::Geo g;
    int rc = setup::read_mesh(p, m, g, err);
    if (rc) return rc;
    setup::cell_geometry(g);
    rc = setup::ghosts_and_pairs(p, g, err);
    if (rc) return rc;
    setup::vertex_weights(g);
    setup::edge_geometry(g);
    return setup::finish_layout(p, g, L, err);
}

// The same setup with its floating-point steps on the current device: the
// same bits (setup_gpu.cu), the topology and table packing on the host.
int build_layout_device(const nsmp_params& p, const nsmp_mesh& m, HostLayout& L, std::string& err) {
    setup::Geo g;
    int rc = setup::read_mesh(p, m, g, err);
    if (rc) return rc;
    rc = setup::device_steps(p, g, err);
    if (rc) return rc;
    return setup::finish_layout(p, g, L, err);
}

}  // namespace nsmp
