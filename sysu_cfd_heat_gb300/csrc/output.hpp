// Output writers of the reference (Tecplot FEBRICK files and tot.dat) from host
// copies of the fields; see output.cpp.
#pragma once

#include <string>

#include "case.hpp"

namespace sysu {

// Cell fields of the fluid in reference cell order; TE, ED only with
// turbulence ke; solid_T only for a conjugate heat transfer case.
struct TecFields {
    const double *P = nullptr, *U = nullptr, *V = nullptr, *W = nullptr, *R = nullptr, *T = nullptr;
    const double *VisLam = nullptr, *VisTur = nullptr, *TE = nullptr, *ED = nullptr;
    const double *solid_T = nullptr;
};

// NavierStokesSolver::Output2Tecplot + the solid zone, to `path` (truncated).
void write_tecplot(const Case &cs, const std::string &path, const TecFields &f);
// tot.dat header (the NavierStokesSolver constructor), truncating `path`.
void write_tot_header(const std::string &path);
// NavierStokesSolver::VolumnAverage: one line appended to `path`.
void append_tot_line(const Case &cs, const std::string &path, double t, int out_iter, const double *R,
                     const double *P, const double *T);

}  // namespace sysu
