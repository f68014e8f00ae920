// ORACLE / TEST INFRASTRUCTURE ONLY -- never part of the product.
//
// Dump driver for the reference solver.  It is linked against the reference's
// own, unmodified src/*.cpp (all but main.cpp) and the CPU LASPack restatement
// in laspack_cpu.c.  It repeats the set-up sequence of main.cpp:8-33
// (ReadParamFile, ReadGridFile, CreateFaces, buildSolver, CellFaceInfo,
// CheckAndAllocate, InitFlowField) and then either
//   * calls NavierStokesSolver::NSSolve() unchanged  (-nssolve), or
//   * runs the body of the NSSolve steady loop (navier.cpp:33-68) for a fixed
//     number of outer iterations, timing each one, and dumps the fields as raw
//     float64 so that other implementations can be compared bit for bit.
//
// Usage: cycas_ref -paramfile <param.in> [-iters N] [-dump DIR] [-geom]
//                  [-stage1 DIR] [-quiet] [-nssolve] [-timing FILE]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <chrono>

#include "BasicType.h"
#include "HeatConductionSolver.h"
#include "PreProcessor.h"
#include "navier.h"

ErrorHandler *errorHandler;  // defined by the reference's main.cpp, which is not linked

#ifdef SYSU_GPU_LASPACK
// linked against the GPU LASPack ABI: no per-iterator timing statistics there
struct LaspackOracleStats {
    long calls[3];
    long iters[3];
    double seconds[3];
};
static LaspackOracleStats g_nostats;
static void laspack_oracle_reset_stats() {}
static const LaspackOracleStats *laspack_oracle_stats() { return &g_nostats; }
#endif

namespace {

std::string g_dump;

void write_raw(const std::string &dir, const std::string &name, const void *p, size_t bytes) {
    std::string path = dir + "/" + name;
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        std::fprintf(stderr, "driver: cannot write %s\n", path.c_str());
        std::exit(4);
    }
    if (bytes) std::fwrite(p, 1, bytes, f);
    std::fclose(f);
}

void dump_vec(const std::string &dir, const std::string &name, const double *p, int n) {
    if (!p) return;
    write_raw(dir, name + ".f64", p, sizeof(double) * (size_t)n);
}

void dump_grad(const std::string &dir, const std::string &name, double **g, int n) {
    if (!g) return;
    std::vector<double> buf((size_t)n * 3);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) buf[(size_t)i * 3 + k] = g[i][k];
    write_raw(dir, name + ".f64", buf.data(), buf.size() * sizeof(double));
}

// Geometry as computed by CycasSolver::CellFaceInfo (BasicSolver.cpp:317-512).
void dump_geometry(const std::string &dir, const std::string &pre, CycasSolver *s) {
    int nc = s->Ncel, nf = s->Nfac, nb = s->Nbnd;
    std::vector<double> cvol(nc), cx((size_t)nc * 3);
    std::vector<int> cnf(nc), cface((size_t)nc * 6, -1), cnbr((size_t)nc * 6, -100), crid(nc),
        cvert((size_t)nc * 8);
    for (int i = 0; i < nc; ++i) {
        cvol[i] = s->Cell[i].vol;
        for (int k = 0; k < 3; ++k) cx[(size_t)i * 3 + k] = s->Cell[i].x[k];
        cnf[i] = s->Cell[i].nface;
        crid[i] = s->Cell[i].rid;
        for (int j = 0; j < s->Cell[i].nface; ++j) {
            cface[(size_t)i * 6 + j] = s->Cell[i].face[j];
            cnbr[(size_t)i * 6 + j] = s->Cell[i].cell[j];
        }
        for (int j = 0; j < 8; ++j) cvert[(size_t)i * 8 + j] = s->Cell[i].vertices[j];
    }
    write_raw(dir, pre + "cell_vol.f64", cvol.data(), cvol.size() * 8);
    write_raw(dir, pre + "cell_x.f64", cx.data(), cx.size() * 8);
    write_raw(dir, pre + "cell_nface.i32", cnf.data(), cnf.size() * 4);
    write_raw(dir, pre + "cell_face.i32", cface.data(), cface.size() * 4);
    write_raw(dir, pre + "cell_nbr.i32", cnbr.data(), cnbr.size() * 4);
    write_raw(dir, pre + "cell_rid.i32", crid.data(), crid.size() * 4);
    write_raw(dir, pre + "cell_vert.i32", cvert.data(), cvert.size() * 4);
    std::vector<double> fx((size_t)nf * 3), fn((size_t)nf * 3), farea(nf), flam(nf), frl(nf),
        fxp((size_t)nf * 3), fxn((size_t)nf * 3);
    std::vector<int> fc1(nf), fc2(nf), fbnd(nf), fvert((size_t)nf * 4);
    for (int i = 0; i < nf; ++i) {
        const FaceData &f = s->Face[i];
        for (int k = 0; k < 3; ++k) {
            fx[(size_t)i * 3 + k] = f.x[k];
            fn[(size_t)i * 3 + k] = f.n[k];
            // Xpac/Xnac are only set for interior faces (BasicSolver.cpp:495-508)
            fxp[(size_t)i * 3 + k] = f.cell2 >= 0 ? f.Xpac[k] : 0.0;
            fxn[(size_t)i * 3 + k] = f.cell2 >= 0 ? f.Xnac[k] : 0.0;
        }
        farea[i] = f.area;
        flam[i] = f.lambda;
        frl[i] = f.rlencos;
        fc1[i] = f.cell1;
        fc2[i] = f.cell2;
        fbnd[i] = f.bnd;
        for (int k = 0; k < 4; ++k) fvert[(size_t)i * 4 + k] = f.vertices[k];
    }
    write_raw(dir, pre + "face_x.f64", fx.data(), fx.size() * 8);
    write_raw(dir, pre + "face_n.f64", fn.data(), fn.size() * 8);
    write_raw(dir, pre + "face_area.f64", farea.data(), farea.size() * 8);
    write_raw(dir, pre + "face_lambda.f64", flam.data(), flam.size() * 8);
    write_raw(dir, pre + "face_rlencos.f64", frl.data(), frl.size() * 8);
    write_raw(dir, pre + "face_xpac.f64", fxp.data(), fxp.size() * 8);
    write_raw(dir, pre + "face_xnac.f64", fxn.data(), fxn.size() * 8);
    write_raw(dir, pre + "face_c1.i32", fc1.data(), fc1.size() * 4);
    write_raw(dir, pre + "face_c2.i32", fc2.data(), fc2.size() * 4);
    write_raw(dir, pre + "face_bnd.i32", fbnd.data(), fbnd.size() * 4);
    write_raw(dir, pre + "face_vert.i32", fvert.data(), fvert.size() * 4);
    std::vector<int> bface(nb), brid(nb);
    std::vector<double> bdist(nb);
    for (int i = 0; i < nb; ++i) {
        bface[i] = s->Bnd[i].face;
        brid[i] = s->Bnd[i].rid;
        bdist[i] = s->Bnd[i].distance;
    }
    write_raw(dir, pre + "bnd_face.i32", bface.data(), bface.size() * 4);
    write_raw(dir, pre + "bnd_rid.i32", brid.data(), brid.size() * 4);
    write_raw(dir, pre + "bnd_distance.f64", bdist.data(), bdist.size() * 8);
}

HeatConductionSolver *solid_of(NavierStokesSolver *ns) {
    if (!ns->Solve3DHeatConduction) return nullptr;
    return dynamic_cast<HeatConductionSolver *>(ns->physicalModule["3dHeatConduction"]);
}

void dump_fields(const std::string &dir, NavierStokesSolver *ns) {
    int n = ns->Ncel;
    dump_vec(dir, "U", ns->Un, n);
    dump_vec(dir, "V", ns->Vn, n);
    dump_vec(dir, "W", ns->Wn, n);
    dump_vec(dir, "P", ns->Pn, n);
    dump_vec(dir, "R", ns->Rn, n);
    dump_vec(dir, "T", ns->Tn, n);
    dump_vec(dir, "TE", ns->TE, n);
    dump_vec(dir, "ED", ns->ED, n);
    dump_vec(dir, "VisTur", ns->VisTur, n);
    dump_vec(dir, "VisLam", ns->VisLam, n);
    dump_vec(dir, "Apr", ns->Apr, n);
    dump_vec(dir, "RUFace", ns->RUFace, ns->Nfac);
    dump_vec(dir, "BU", ns->BU, ns->Nbnd);
    dump_vec(dir, "BV", ns->BV, ns->Nbnd);
    dump_vec(dir, "BW", ns->BW, ns->Nbnd);
    dump_vec(dir, "BRo", ns->BRo, ns->Nbnd);
    dump_vec(dir, "BPre", ns->BPre, ns->Nbnd);
    dump_vec(dir, "BTem", ns->BTem, ns->Nbnd);
    dump_vec(dir, "BTE", ns->BTE, ns->Nbnd);
    dump_vec(dir, "BED", ns->BED, ns->Nbnd);
    dump_grad(dir, "dUdX", ns->dUdX, n);
    dump_grad(dir, "dVdX", ns->dVdX, n);
    dump_grad(dir, "dWdX", ns->dWdX, n);
    dump_grad(dir, "dPdX", ns->dPdX, n);
    dump_grad(dir, "dPhidX", ns->dPhidX, n);
    std::vector<double> bq(ns->Nbnd);
    for (int i = 0; i < ns->Nbnd; ++i) bq[i] = ns->Bnd[i].q;
    write_raw(dir, "Bq.f64", bq.data(), bq.size() * 8);
    HeatConductionSolver *ht = solid_of(ns);
    if (ht) {
        dump_vec(dir, "solid_T", ht->Tn, ht->Ncel);
        dump_vec(dir, "solid_BTem", ht->BTem, ht->Nbnd);
        dump_grad(dir, "solid_dPhidX", ht->dPhidX, ht->Ncel);
        std::vector<double> sq(ht->Nbnd);
        for (int i = 0; i < ht->Nbnd; ++i) sq[i] = ht->Bnd[i].q;
        write_raw(dir, "solid_Bq.f64", sq.data(), sq.size() * 8);
    }
    FILE *f = std::fopen((dir + "/meta.txt").c_str(), "w");
    if (f) {
        std::fprintf(f, "Ncel %d\nNfac %d\nNbnd %d\nNvrt %d\nNCoupledBnd %d\n", ns->Ncel, ns->Nfac,
                     ns->Nbnd, ns->Nvrt, ns->NCoupledBnd);
        std::fprintf(f, "TurModel %d\nSolveEnergy %d\nSolve3DHeatConduction %d\nlimiter %d\n",
                     ns->TurModel, (int)ns->SolveEnergy, (int)ns->Solve3DHeatConduction, ns->limiter);
        std::fprintf(f, "cellPressureRef %d\n", ns->cellPressureRef);
        if (ht)
            std::fprintf(f, "solid_Ncel %d\nsolid_Nfac %d\nsolid_Nbnd %d\nsolid_NCoupledBnd %d\n",
                         ht->Ncel, ht->Nfac, ht->Nbnd, ht->NCoupledBnd);
        std::fclose(f);
    }
}

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char **argv) {
    int iters = -1;
    bool quiet = false, geom = false, nssolve = false;
    std::string stage1, timing;
    std::vector<char *> passthru;
    passthru.push_back(argv[0]);
    for (int i = 1; i < argc; ++i) {
        std::string a(argv[i]);
        if (a == "-iters" && i + 1 < argc) iters = std::atoi(argv[++i]);
        else if (a == "-dump" && i + 1 < argc) g_dump = argv[++i];
        else if (a == "-stage1" && i + 1 < argc) stage1 = argv[++i];
        else if (a == "-timing" && i + 1 < argc) timing = argv[++i];
        else if (a == "-geom") geom = true;
        else if (a == "-quiet") quiet = true;
        else if (a == "-nssolve") nssolve = true;
        else passthru.push_back(argv[i]);
    }
    if (quiet) {
        if (!std::freopen("/dev/null", "w", stdout)) return 5;
    }
    double t_setup0 = now_s();
    // --- main.cpp:14-28, unchanged order ---
    errorHandler = new ErrorHandler;
    NavierStokesSolver *ns = new NavierStokesSolver;
    PreProcessor *pre = new PreProcessor;
    pre->parseCommandLine((int)passthru.size(), passthru.data());
    pre->ReadParamFile(ns);
    pre->ReadGridFile();
    pre->CreateFaces();
    pre->buildSolver(ns);
    ns->CellFaceInfo();
    ns->CheckAndAllocate();
    ns->InitFlowField();
    delete pre;
    double t_setup1 = now_s();
    HeatConductionSolver *ht = solid_of(ns);

    if (geom && !g_dump.empty()) {
        dump_geometry(g_dump, "", ns);
        if (ht) dump_geometry(g_dump, "solid_", ht);
    }

    FILE *tf = timing.empty() ? nullptr : std::fopen(timing.c_str(), "w");
    if (tf) {
        std::fprintf(tf, "setup_s %.6f\n", t_setup1 - t_setup0);
        std::fflush(tf);
    }

    int done = 0;
    if (nssolve) {
        double t0 = now_s();
        ns->NSSolve();
        double t1 = now_s();
        if (tf) std::fprintf(tf, "nssolve_s %.6f\n", t1 - t0);
    } else {
        if (iters < 0) iters = ns->MaxStep - 1;  // "steady, N" runs N-1 outer iterations
        FILE *rf = g_dump.empty() ? nullptr : std::fopen((g_dump + "/iters.txt").c_str(), "w");
        for (int it = 1; it <= iters; ++it) {
            laspack_oracle_reset_stats();
            double t0 = now_s();
            // navier.cpp:36-53, the body of the steady outer loop
            ns->CalculateVelocity();
            double t1 = now_s();
            if (it == 1 && !stage1.empty()) {
                std::string d = stage1;
                dump_grad(d, "dUdX", ns->dUdX, ns->Ncel);
                dump_grad(d, "dVdX", ns->dVdX, ns->Ncel);
                dump_grad(d, "dWdX", ns->dWdX, ns->Ncel);
                dump_grad(d, "dPdX", ns->dPdX, ns->Ncel);
                dump_vec(d, "Apr", ns->Apr, ns->Ncel);
                dump_vec(d, "Ustar", ns->Un, ns->Ncel);
                dump_vec(d, "Vstar", ns->Vn, ns->Ncel);
                dump_vec(d, "Wstar", ns->Wn, ns->Ncel);
                // Rhie-Chow fluxes of the predicted velocity; CalculatePressure
                // recomputes exactly these (navier_pressure.cpp:83-84).
                ns->SetBCVelocity(ns->BRo, ns->BU, ns->BV, ns->BW);
                ns->CalRUFace2();
                dump_vec(d, "RUFace_star", ns->RUFace, ns->Nfac);
                dump_vec(d, "BU", ns->BU, ns->Nbnd);
                dump_vec(d, "BV", ns->BV, ns->Nbnd);
                dump_vec(d, "BW", ns->BW, ns->Nbnd);
            }
            double t2 = now_s();
            ns->CalculatePressure();
            double t3 = now_s();
            if (it == 1 && !stage1.empty()) {
                std::string d = stage1;
                dump_vec(d, "dp", ns->xsol.Cmp + 1, ns->Ncel);
                dump_grad(d, "dPdX_dp", ns->dPdX, ns->Ncel);
                dump_vec(d, "P1", ns->Pn, ns->Ncel);
                dump_vec(d, "U1", ns->Un, ns->Ncel);
                dump_vec(d, "V1", ns->Vn, ns->Ncel);
                dump_vec(d, "W1", ns->Wn, ns->Ncel);
                dump_vec(d, "RUFace1", ns->RUFace, ns->Nfac);
            }
            if (ns->TurModel == 1) ns->UpdateTurKEpsilon();
            double t4 = now_s();
            if (ns->SolveEnergy) {
                ns->UpdateEnergy();
                if (ht) ht->solve();
            }
            double t5 = now_s();
            double resmax = vec_max(ns->Residual, 10);
            const LaspackOracleStats *st = laspack_oracle_stats();
            if (rf)
                std::fprintf(rf, "%d %.17g %.17g %.17g %.17g %.17g\n", it, ns->Residual[0], ns->Residual[1],
                             ns->Residual[2], ns->Residual[3], resmax);
            if (tf)
                std::fprintf(tf, "iter %d total_s %.6f mom_s %.6f p_s %.6f ke_s %.6f energy_s %.6f "
                                 "cg_s %.6f bicgstab_s %.6f gmres_s %.6f cg_it %ld bicgstab_it %ld gmres_it %ld\n",
                             it, t5 - t0 - (t2 - t1), t1 - t0, t3 - t2, t4 - t3, t5 - t4, st->seconds[0],
                             st->seconds[1], st->seconds[2], st->iters[0], st->iters[1], st->iters[2]);
            if (tf) std::fflush(tf);  // a caller may stop the run between iterations
            ++done;
            if (ns->IfSteady && resmax < ns->ResidualSteady) break;  // navier.cpp:68
        }
        if (rf) std::fclose(rf);
    }
    if (tf) std::fclose(tf);
    if (!g_dump.empty()) dump_fields(g_dump, ns);
    std::fprintf(stderr, "driver: %d outer iterations done\n", done);
    // main.cpp ends without deleting the solver, which leaves the buffered tail
    // of tot.dat unwritten; after NSSolve the driver flushes the (public) stream
    // the destructor would close (navier.cpp:420-432)
    if (nssolve) ns->totFile.flush();
    return 0;
}
