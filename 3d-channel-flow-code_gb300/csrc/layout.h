// Device data layout of the nsmp3D hot path and the host-side setup that
// produces it.
//
// Layout in HBM:
//  * a cell field is N0 sigma columns x NZ layers, layer fastest:
//    f[c*NZ + k0], k0 = 0..NZ-1 (k0 = 0 and NZ-1 are the wall ghost layers,
//    i.e. the reference's k = 1 and k = NZ).  Columns are the interior
//    triangles renumbered by reverse Cuthill-McKee; lateral ghost cells do
//    not exist on the device because every lateral ghost of the supported
//    configuration is a periodic copy (BC.F90:540-581, flag 3) and is
//    resolved into the neighbour index of the periodic image.
//  * a vertex field holds one value per periodic vertex class (copies of a
//    boundary vertex merged, as bc_periodic averages them) and interior layer:
//    fv[v*NZI + k0-1], NZI = NZ-2.
//  * per-column coefficients are small structs (one warp reads one or two
//    columns, so the loads broadcast); per-layer factors are short arrays.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "nsmp.h"

namespace nsmp {

// Coefficients of one column used by the matrix-free PPE operator
// (PDE.F90:69-121): AA_j = kA_j * dsigv(k-1), AAB/AAT = area / dsig.
struct ColPPE {
    int nb[3];
    int pad;
    double kA[3];
    double area;
};

// FP32 copy of ColPPE for the mixed-precision inner solver.
struct ColPPE32 {
    int nb[3];
    float kA[3];
    float area;
    float pad;
};

// Coefficients of one column used by the stage kernels.
struct ColGeo {
    int nb[3];       // neighbour column across edge j
    int vtx[3];      // vertex class of vertex j (edge j joins vtx[j], vtx[j+1])
    double kA[3];    // dle1/dlCC*dlVV      (diffusion flux, PPE)
    double dle2[3];  // dle2                (cross diffusion x dlVV/dlVV)
    double cA[3];    // dle1/dlCC           (newu3D principal)
    double cB[3];    // dle2/dlVV           (newu3D cross)
    double kE[3];    // doe/dlVV            (calcul_face Kim-Choi correction)
    double L[3];     // dlVV
    double xn[3], yn[3];  // outward unit normals
    double gx[3], gy[3];  // LSQ gradient weights (gradientLSM.F90:153-168)
    double lxu[3], lyu[3];  // FVM gradient weights xnn*dlVV/area (u, w)
    double lxv[3], lyv[3];  // same for v (reference pairs faces 2/3 with dlVV 3/2)
    double area, inv_area, cbrt_area;
    int bnd;         // bit j set: edge j is a lateral boundary edge (a ghost in the reference)
    int orig;        // original (data.txt) cell number, 0-based
};

// FP32 copy of the ColGeo members the stage right-hand side reads (the FP32
// stage arithmetic of the mixed form).
struct ColGeo32 {
    int nb[3];
    int vtx[3];
    float kA[3], dle2[3], kE[3], L[3];
    float lxu[3], lyu[3], lxv[3], lyv[3];
    float area, inv_area, cbrt_area, pad;
};

// Per-layer factors, indexed by k0 = 1..NZ-2 (entries 0 and NZ-1 unused).
struct Levels {
    std::vector<double> dsv;     // dsigv(k-1)
    std::vector<double> idsT;    // 1/dsig(k)
    std::vector<double> idsB;    // 1/dsig(k-1)
    std::vector<double> idsBu;   // bottom face divisor of newu3D (1/dsig(k) as shipped)
    std::vector<double> wT, wB;  // 1 or 0: PPE top/bottom coupling (0 at the walls)
    std::vector<double> gzp, gzm;// vertical LSQ weights dzp/S, dzm/S
    std::vector<double> hmean;   // Glob_Norm layer weight
    std::vector<double> les_dd;  // Cs*dsig(k)^(1/3)
    std::vector<double> les_kd;  // von_Karman*walld
    std::vector<double> les_damp;// 1-exp(-walld*Re/A+)
    std::vector<double> ihz;     // 1/dz of the FVM vertical gradient
    std::vector<double> cfl_div; // glob_cfl lateral-flux height: dsig(k-1) as shipped (cfl.F90:139)
    std::vector<double> cfl_h;   // glob_cfl CFL / mean / side-flux height: dsig(k) as shipped (cfl.F90:140,161)
};

struct HostLayout {
    int N0 = 0, NV = 0, NZ = 0, NZI = 0, NC = 0, nclass = 0;
    double total_volume = 0.0, lsig = 0.0;
    std::vector<int> perm;       // new column -> original cell (0-based)
    std::vector<int> iperm;      // original cell -> new column
    std::vector<int> ghost_img;  // ghost g (reference number N0+1+g) -> image cell (0-based)
    std::vector<int> vclass;     // reference vertex (0-based) -> class
    std::vector<ColPPE> ppe;
    std::vector<ColGeo> geo;
    std::vector<int> vptr;       // class stencil CSR
    std::vector<int> vcell;
    std::vector<double> vcoef;
    Levels lev;
    std::vector<double> sig, dsig, sigv, dsigv;
    double sgn_bot[3], sgn_top[3];  // wall ghost sign of u, v, w
    // Reference-shaped geometry kept for diagnostics (Fortran layout).
    std::vector<double> ref_xc, ref_yc, ref_area;   // (N_CELL)
    std::vector<double> ref_dlVV, ref_dlCC, ref_dle1, ref_dle2, ref_doe, ref_xnn, ref_ynn,
        ref_dxCC, ref_dyCC;                          // (N0,3)
    std::vector<double> ref_sxx, ref_syy, ref_sxy;  // (N0)
    std::vector<double> ref_dlVsum;                 // (N_VERT)
    std::vector<int> ref_No_cp;                     // (N_CELL,3)
};

// Builds the geometry and the device tables; returns 0 or an NSMP_ERR code
// with a message in err.
int build_layout(const nsmp_params& p, const nsmp_mesh& m, HostLayout& out, std::string& err);
// The same tables, with the floating-point geometry computed on the current
// device (bit-identical to build_layout; needs a GPU).
int build_layout_device(const nsmp_params& p, const nsmp_mesh& m, HostLayout& out, std::string& err);

}  // namespace nsmp
