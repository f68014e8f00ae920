// Output writers of the reference, from host copies of the fields:
//   Tecplot FEBRICK block files  NavierStokesSolver::Output / Output2Tecplot
//                                (navier.cpp:264-337) with the solid zone of
//                                HeatConductionSolver::Output2Tecplot
//                                (HeatConductionSolver.cpp:330-361)
//   tot.dat                      header (navier.cpp:413-415) and one
//                                VolumnAverage line per time step
//                                (navier.cpp:243-261)
// The text is byte-for-byte the reference's: numbers go through the default
// formatting of std::ostream (printf "%g", 6 significant digits), with the
// reference's separators, line breaks every five values and its header quirks
// (no comma between "z" and "p", none before DATAPACKING).
#include "output.hpp"

#include <cmath>
#include <cstdio>
#include <fstream>

namespace sysu {
namespace {

struct Text {
    std::string s;
    char buf[64];
    void num(double v) {
        int k = std::snprintf(buf, sizeof buf, "%g", v);
        s.append(buf, (size_t)k);
    }
    void inum(long v) {
        int k = std::snprintf(buf, sizeof buf, "%ld", v);
        s.append(buf, (size_t)k);
    }
    void str(const char *t) { s += t; }
    void nl() { s += '\n'; }
};

// tools.cpp:74-81 (two spaces after every value)
void out_array(Text &t, const double *a, int n) {
    for (int i = 0; i < n; ++i) {
        t.num(a[i]);
        t.str("  ");
        if (i % 5 == 4) t.nl();
    }
    t.nl();
}

// tools.cpp:66-72 (one space)
void out_placeholder(Text &t, double v, int n) {
    for (int i = 0; i < n; ++i) {
        t.num(v);
        t.str(" ");
        if (i % 5 == 4) t.nl();
    }
    t.nl();
}

void zone_head(Text &t, const Domain &d, int nvar) {
    t.str("zone n=");
    t.inum(d.nv);
    t.str(", e=");
    t.inum(d.nc);
    t.str(", VARLOCATION=([1-3]=NODAL,[4-");
    t.inum(nvar);
    t.str("]=CELLCENTERED)DATAPACKING=BLOCK, ZONETYPE=FEBRICK");
    t.nl();
    for (int j = 0; j < 3; ++j) {
        for (int i = 0; i < d.nv; ++i) {
            t.num(d.vert[3 * (size_t)i + j]);
            t.str(" ");
            if (i % 5 == 4) t.nl();
        }
        t.nl();
    }
}

void connectivity(Text &t, const Domain &d) {
    for (int i = 0; i < d.nc; ++i) {
        for (int j = 0; j < 8; ++j) {
            t.inum(d.cell_vert[8 * (size_t)i + j] + 1);
            t.str(" ");
        }
        t.nl();
    }
}

void write_file(const std::string &path, const std::string &text, bool append) {
    std::ofstream of(path, append ? std::ios::app : std::ios::trunc);
    if (!of) throw CaseError{"cannot open " + path + " for writing"};
    of.write(text.data(), (std::streamsize)text.size());
    if (!of) throw CaseError{"write failed: " + path};
}

}  // namespace

void write_tecplot(const Case &cs, const std::string &path, const TecFields &f) {
    const Params &p = cs.params;
    const Domain &d = cs.fluid;
    const int n = d.nc;
    for (const double *a : {f.P, f.U, f.V, f.W, f.R, f.T, f.VisLam, f.VisTur})
        if (!a) throw CaseError{"write_tecplot: P U V W R T VisLam VisTur are required"};
    const bool ke = p.tur_model == 1;
    if (ke && (!f.TE || !f.ED)) throw CaseError{"write_tecplot: TE and ED are required with turbulence ke"};
    if (cs.has_solid && !f.solid_T) throw CaseError{"write_tecplot: solid_T is required for the solid zone"};
    Text t;
    t.s.reserve((size_t)n * 200 + (size_t)d.nv * 40);
    t.str("variables=\"x\",\"y\",\"z\"\"p\",\"u\",\"v\",\"w\",\"ro\",\"T\",\"Mach\",\"mu\"");
    int nvar = 11;
    if (ke) {
        t.str("\"te\"\"ed\"");
        nvar = 13;
    }
    t.nl();
    zone_head(t, d, nvar);
    out_array(t, f.P, n);
    out_array(t, f.U, n);
    out_array(t, f.V, n);
    out_array(t, f.W, n);
    out_array(t, f.R, n);
    out_array(t, f.T, n);
    std::vector<double> tmp((size_t)n);
    for (int i = 0; i < n; ++i) {  // Mach / velocity magnitude
        double u2 = f.U[i] * f.U[i] + f.V[i] * f.V[i] + f.W[i] * f.W[i];
        tmp[i] = p.density_model == 1 ? std::sqrt(u2 / (p.gama * (f.P[i] + p.pressure_reference) / f.R[i]))
                                      : std::sqrt(u2);
    }
    out_array(t, tmp.data(), n);
    for (int i = 0; i < n; ++i) tmp[i] = f.VisLam[i] + f.VisTur[i];
    out_array(t, tmp.data(), n);
    if (ke) {
        out_array(t, f.TE, n);
        out_array(t, f.ED, n);
    }
    connectivity(t, d);
    if (cs.has_solid) {
        const Domain &s = cs.solid;
        zone_head(t, s, nvar);
        for (int k = 0; k < 5; ++k) out_placeholder(t, 0.0, s.nc);
        out_array(t, f.solid_T, s.nc);
        for (int k = 10; k != nvar + 1; ++k) out_placeholder(t, 0.0, s.nc);
        connectivity(t, s);
    }
    write_file(path, t.s, false);
}

void write_tot_header(const std::string &path) {
    char buf[256];
    std::snprintf(buf, sizeof buf, "%20s %20s %20s %20s %20s\n", "time", "outIter", "Ro", "P", "T");
    write_file(path, buf, false);
}

void append_tot_line(const Case &cs, const std::string &path, double t, int out_iter, const double *R,
                     const double *P, const double *T) {
    const Domain &d = cs.fluid;
    double avg[3] = {0.0, 0.0, 0.0}, sumvol = 0.0;
    for (int i = 0; i < d.nc; ++i) {
        double vol = d.cell_vol[i];
        sumvol += vol;
        avg[0] += R[i] * vol;
        avg[1] += P[i] * vol;
        avg[2] += T[i] * vol;
    }
    for (double &a : avg) a /= sumvol;
    char buf[256];
    std::snprintf(buf, sizeof buf, "%20e %20d %20e %20e %20e\n", t, out_iter, avg[0], avg[1], avg[2]);
    write_file(path, buf, true);
}

}  // namespace sysu
