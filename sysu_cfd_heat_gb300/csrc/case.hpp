// Host-side case description: parameters (param.in), mesh topology and
// finite-volume geometry, laid out as structure-of-arrays ready for upload.
//
// Reference semantics followed here:
//   parameters  readparamfile.cpp:10-260, navier.cpp:354-416 (defaults)
//   mesh input  Preprocessor.cpp:13-146 (Gmsh MSH 2.x ASCII)
//   faces       Preprocessor.cpp:181-299 (CreateFaces / FindFace order)
//   CHT split   Preprocessor.cpp:308-515 (findCoupledBoundary / buildSolver)
//   geometry    BasicSolver.cpp:317-512 (CellFaceInfo)
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace sysu {

// Boundary/volume region, BasicType.h:69-95.
struct Region {
    std::string name;
    int type1 = -1;  // 1 wall, 2 inlet, 3 outlet, 4 symmetry, 5 body
    int type2 = -1;  // wall: 0 fixed T, 1 fixed flux, 2 coupled; body: 0 fluid, 1 solid
    double fixedValue = 2147483647.0;  // CYCASHUGE_I
    double initvalues[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
};

struct Params {
    std::string gridfile;
    bool steady = true;
    double dt = 0.0, total_time = 0.0;
    int time_scheme = 1;
    int max_step = 10000;
    int max_outer_step = 50;
    double residual_steady = 1e-6;
    bool solve_energy = false;
    bool solve_species = false;
    bool heat_conduction = false;
    int density_model = 0;
    int tur_model = 0;
    double gravity[3] = {0, 0, 0};
    double pressure_reference = 1.01325e5;
    int cell_pressure_ref = 0;
    double urf[8] = {0.6, 0.6, 0.6, 0.5, 0.8, 0.8, 0.8, 0.8};
    int limiter = 0;  // 0 none, 1 Barth, 2 MLP, 3 WENO
    std::vector<double> initflow;
    bool has_initflow = false;
    int noutput = 1;
    int outputformat = 0;
    std::map<int, Region> regions;
    // material constants of NavierStokesSolver (navier.cpp:376-383); no keyword sets them
    double gama = 1.4, cp = 1006.0, prl = 0.72, prte = 0.9, temp_ref = 273.15;
    double cv() const { return cp / gama; }
    double rcpcv() const { return cp - cp / gama; }
};

// Mesh as read: every cell as an 8-vertex hexahedron (Preprocessor.cpp:97-133),
// every boundary element as a 4-vertex face.
struct RawMesh {
    int nv = 0;
    std::vector<double> vert;      // 3*nv
    std::vector<int> cell_vert;    // 8*nc
    std::vector<int> cell_rid;
    std::vector<int> bnd_vert;     // 4*nb
    std::vector<int> bnd_rid;
    int ncell() const { return (int)cell_rid.size(); }
    int nbnd() const { return (int)bnd_rid.size(); }
};

// Topology + geometry of one domain (the fluid, or the solid of a CHT case),
// indexed exactly like the reference (face ids, boundary ids, cell ids).
struct Domain {
    int nv = 0, nc = 0, nf = 0, nb = 0, ncb = 0;  // ncb: first coupled boundary record
    std::vector<double> vert;                      // 3*nv
    // cells
    std::vector<int> cell_vert;   // 8*nc
    std::vector<int> cell_rid;
    std::vector<int> cell_nface;
    std::vector<int> cell_face;   // 6*nc (reference Cell[i].face[j])
    std::vector<int> cell_nbr;    // 6*nc (Cell[i].cell[j], <0 on boundary)
    std::vector<double> cell_vol, cell_x;  // nc, 3*nc
    // faces
    std::vector<int> face_vert;   // 4*nf
    std::vector<int> face_c1, face_c2, face_bnd;
    std::vector<double> face_x, face_n, face_area, face_lambda, face_rlencos, face_xpac, face_xnac;
    // boundary records
    std::vector<int> bnd_face, bnd_rid;
    std::vector<double> bnd_distance;
};

struct Case {
    Params params;
    Domain fluid;
    Domain solid;
    bool has_solid = false;
    int coupled_rid = -1;
};

// Errors are reported through this exception inside the library and turned
// into status codes + messages at the C ABI.
struct CaseError {
    std::string msg;
};

Params parse_params(const std::string &path);
RawMesh read_msh(const std::string &path);
// Wall-clock seconds of the last preprocessing on this thread: [0] MSH read,
// [1] face construction, [2] fluid/solid split, [3] geometry; threads used in [4].
double *setup_phases();
// CreateFaces + (optional) fluid/solid split + CellFaceInfo.
void build_case(const RawMesh &raw, Case &cs);
void cell_face_info(Domain &d);

}  // namespace sysu
