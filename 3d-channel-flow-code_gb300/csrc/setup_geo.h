// The setup's intermediate geometry (calcul_geometry.F90 arrays, 0-based)
// and its steps, shared by the host path (setup.cpp) and the device path of
// the floating-point steps (setup_gpu.cu).
#pragma once
#include <string>
#include <utility>
#include <vector>

#include "layout.h"

namespace nsmp {
namespace setup {

struct Geo {
    int N0, NV, NZ, NC;
    // mesh (0-based copies)
    std::vector<int> vp;   // (N0,3): vertex (0-based)
    std::vector<int> cp;   // (NCmax,3): neighbour (0-based, -1 = none)
    std::vector<int> nbe, nbev;
    std::vector<double> xv, yv;
    // geometry
    std::vector<double> xc, yc, area;                 // (NC)
    std::vector<double> dxVV, dyVV, dlVV, xnn, ynn;   // (N0,3)
    std::vector<double> dxCC, dyCC, dlCC, dle1, dle2, doe;
    std::vector<double> sxx, syy, sxy;
    std::vector<int> img;                             // ghost -> image cell (0-based)
    std::vector<std::vector<std::pair<int, double>>> stencil;  // per vertex: (cell, weight)
    std::vector<double> dlVsum;
    std::vector<int> vpair, vedge;
    double total_volume = 0.0;
    int at(int i, int j) const { return i + j * N0; }
};


// Steps of the setup.  The floating-point ones (cell_geometry,
// vertex_weights, edge_geometry) have device counterparts in setup_gpu.cu
// that compute the same bits; the topology steps stay on the host.
int read_mesh(const nsmp_params& p, const nsmp_mesh& m, Geo& g, std::string& err);
void cell_geometry(Geo& g);                                          // calcul_geometry.F90:292-367
int ghosts_and_pairs(const nsmp_params& p, Geo& g, std::string& err); // :402-578, :893-1040
void vertex_incidence(const Geo& g, std::vector<int>& ptr, std::vector<int>& inc);
void vertex_weights(Geo& g);                                         // :1055-1076
void edge_geometry(Geo& g);                                          // :1343-1387, :1460-1517
int finish_layout(const nsmp_params& p, Geo& g, HostLayout& L, std::string& err);
// The three floating-point steps on the current device (setup_gpu.cu).
int device_steps(const nsmp_params& p, Geo& g, std::string& err);

}  // namespace setup
}  // namespace nsmp
