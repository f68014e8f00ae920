// Host orchestration of the GPU SIMPLE iteration.  Every piece is enqueued on
// one stream; the only host synchronisation per outer iteration is the read
// of the residual monitor and the solve status words in check_iteration().
#include "solver.hpp"
#include "graph_loop.hpp"

#include <sys/stat.h>

#include "output.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace sysu {

namespace {
constexpr double SMALL = 1.e-16;
constexpr double CMU = 0.09;  // navier.h:130
}  // namespace

void DomainDev::build(const Domain &d, const Params &p, cudaStream_t st) {
    nc = d.nc;
    nf = d.nf;
    B = d.nb;
    ncb = d.ncb;
    nv = d.nv;
    int2ref.clear();
    for (int f = 0; f < nf; ++f)
        if (d.face_c2[f] >= 0) int2ref.push_back(f);
    F = (int)int2ref.size();
    for (int b = 0; b < B; ++b) int2ref.push_back(d.bnd_face[b]);
    if ((int)int2ref.size() != nf) throw CaseError{"faces without a boundary record"};
    ref2int.assign(nf, -1);
    for (int i = 0; i < nf; ++i) ref2int[int2ref[i]] = i;
    for (int i = 0; i < nf; ++i)
        if (ref2int[i] < 0) throw CaseError{"face permutation is not one to one"};

    std::vector<int> h_fc1(nf), h_fc2(nf);
    std::vector<double> h_fn(3 * (size_t)nf), h_farea(nf), h_flam(nf), h_frl(nf), h_fx(3 * (size_t)nf),
        h_xp(3 * (size_t)std::max(F, 1)), h_xn(3 * (size_t)std::max(F, 1));
    for (int fi = 0; fi < nf; ++fi) {
        int r = int2ref[fi];
        h_fc1[fi] = d.face_c1[r];
        h_fc2[fi] = fi < F ? d.face_c2[r] : -1;
        for (int k = 0; k < 3; ++k) {
            h_fn[(size_t)k * nf + fi] = d.face_n[(size_t)r * 3 + k];
            h_fx[(size_t)k * nf + fi] = d.face_x[(size_t)r * 3 + k];
            if (fi < F) {
                h_xp[(size_t)k * F + fi] = d.face_xpac[(size_t)r * 3 + k];
                h_xn[(size_t)k * F + fi] = d.face_xnac[(size_t)r * 3 + k];
            }
        }
        h_farea[fi] = d.face_area[r];
        h_flam[fi] = d.face_lambda[r];
        h_frl[fi] = d.face_rlencos[r];
    }
    std::vector<double> h_cx(3 * (size_t)nc);
    for (int i = 0; i < nc; ++i)
        for (int k = 0; k < 3; ++k) h_cx[(size_t)k * nc + i] = d.cell_x[(size_t)i * 3 + k];
    std::vector<int> h_csptr(nc + 1, 0), h_csface, h_csk, rowptr(nc + 1, 0), cols;
    h_csface.reserve((size_t)nc * 6);
    h_csk.reserve((size_t)nc * 6);
    cols.reserve((size_t)nc * 7);
    for (int i = 0; i < nc; ++i) {
        cols.push_back(i);
        int k = 1;
        for (int j = 0; j < d.cell_nface[i]; ++j) {
            int r = d.cell_face[(size_t)i * 6 + j];
            int fi = ref2int[r];
            h_csface.push_back(fi);
            if (fi < F) {
                h_csk.push_back(k++);
                int nb_ = d.face_c1[r] == i ? d.face_c2[r] : d.face_c1[r];
                cols.push_back(nb_);
            } else {
                h_csk.push_back(fi - F);
            }
        }
        h_csptr[i + 1] = (int)h_csface.size();
        rowptr[i + 1] = (int)cols.size();
    }
    pat = make_sell(nc, rowptr, cols);
    A.upload(pat, st);
    d_int2ref.upload(int2ref, st);
    {
        // cell slots in SELL-32 layout (fv.hpp: ss_*)
        int nsl = (nc + 31) / 32;
        std::vector<int> sp(nsl + 1, 0), sw(nsl, 0);
        for (int sl = 0; sl < nsl; ++sl) {
            int w = 0;
            for (int i = sl * 32; i < std::min(nc, sl * 32 + 32); ++i) w = std::max(w, h_csptr[i + 1] - h_csptr[i]);
            sw[sl] = w;
            sp[sl + 1] = sp[sl] + 32 * w;
        }
        std::vector<int> sf(std::max(sp[nsl], 1), -1), sn(std::max(sp[nsl], 1), 0);
        for (int i = 0; i < nc; ++i) {
            int sl = i >> 5, lane = i & 31;
            for (int j = 0; j < h_csptr[i + 1] - h_csptr[i]; ++j) {
                int fi = h_csface[h_csptr[i] + j];
                int pos = sp[sl] + 32 * j + lane;
                sf[pos] = fi;
                if (fi < F) {
                    int c1 = h_fc1[fi], c2 = h_fc2[fi];
                    sn[pos] = c1 == i ? c2 : (c1 | SS_C2);
                } else {
                    sn[pos] = SS_BND | (fi - F);
                }
            }
        }
        ss_ptr.upload(sp, st);
        ss_w.upload(sw, st);
        ss_f.upload(sf, st);
        ss_n.upload(sn, st);
    }

    h_bcell.assign(B, 0);
    h_btype1.assign(B, 0);
    h_btype2.assign(B, 0);
    std::vector<int> h_brid(B);
    std::vector<double> h_bdist(B), h_bquirk(B), h_bin(8 * (size_t)std::max(B, 1)), h_bfixed(B);
    has_outlet = false;
    for (int b = 0; b < B; ++b) {
        int r = d.bnd_face[b];
        h_bcell[b] = d.face_c1[r];
        auto it = p.regions.find(d.bnd_rid[b]);
        if (it == p.regions.end()) throw CaseError{"boundary record with an unknown region id"};
        const Region &rg = it->second;
        h_btype1[b] = rg.type1;
        h_btype2[b] = rg.type2;
        h_brid[b] = d.bnd_rid[b];
        h_bdist[b] = d.bnd_distance[b];
        h_bquirk[b] = b < nf ? d.face_area[b] : 0.0;
        for (int k = 0; k < 8; ++k) h_bin[(size_t)k * B + b] = rg.initvalues[k];
        h_bfixed[b] = rg.fixedValue;
        if (rg.type1 == 3) has_outlet = true;
    }
    std::vector<int> h_cwptr(nc + 1, 0), h_cwb;
    {
        std::vector<std::vector<int>> lists(nc);
        for (int b = 0; b < B; ++b)
            if (h_btype1[b] == 1) lists[h_bcell[b]].push_back(b);
        for (int i = 0; i < nc; ++i) {
            h_cwb.insert(h_cwb.end(), lists[i].begin(), lists[i].end());
            h_cwptr[i + 1] = (int)h_cwb.size();
        }
    }
    std::vector<int> h_cvert(8 * (size_t)nc), h_vcptr(nv + 1, 0), h_vccell;
    for (int i = 0; i < nc; ++i)
        for (int k = 0; k < 8; ++k) {
            int v = d.cell_vert[(size_t)i * 8 + k];
            h_cvert[(size_t)k * nc + i] = v;
            h_vcptr[v + 1]++;
        }
    for (int v = 0; v < nv; ++v) h_vcptr[v + 1] += h_vcptr[v];
    h_vccell.assign(h_vcptr[nv], 0);
    {
        std::vector<int> fill(h_vcptr.begin(), h_vcptr.end() - 1);
        for (int i = 0; i < nc; ++i)
            for (int k = 0; k < 8; ++k) h_vccell[fill[d.cell_vert[(size_t)i * 8 + k]]++] = i;
    }

    vol.upload(d.cell_vol, st);
    cx.upload(h_cx, st);
    fn.upload(h_fn, st);
    farea.upload(h_farea, st);
    flam.upload(h_flam, st);
    frl.upload(h_frl, st);
    fx.upload(h_fx, st);
    fxpac.upload(h_xp, st);
    fxnac.upload(h_xn, st);
    {
        std::vector<double> h_d12(std::max(F, 1), 0.0);
        for (int fi = 0; fi < F; ++fi) {
            double dx0 = h_xn[fi] - h_xp[fi], dx1 = h_xn[(size_t)F + fi] - h_xp[(size_t)F + fi],
                   dx2 = h_xn[2 * (size_t)F + fi] - h_xp[2 * (size_t)F + fi];
            h_d12[fi] = std::sqrt(dx0 * dx0 + dx1 * dx1 + dx2 * dx2);
        }
        fd12.upload(h_d12, st);
    }
    bdist.upload(h_bdist, st);
    bquirk.upload(h_bquirk, st);
    bin.upload(h_bin, st);
    bfixed.upload(h_bfixed, st);
    vx.upload(d.vert, st);
    cs_ptr.upload(h_csptr, st);
    cs_face.upload(h_csface, st);
    cs_k.upload(h_csk, st);
    fc1.upload(h_fc1, st);
    fc2.upload(h_fc2, st);
    bcell.upload(h_bcell, st);
    btype1.upload(h_btype1, st);
    btype2.upload(h_btype2, st);
    brid.upload(h_brid, st);
    cw_ptr.upload(h_cwptr, st);
    cw_b.upload(h_cwb, st);
    cvert.upload(h_cvert, st);
    vc_ptr.upload(h_vcptr, st);
    vc_cell.upload(h_vccell, st);

    DomView &v = view;
    v.nc = nc; v.nf = nf; v.F = F; v.B = B; v.ncb = ncb; v.nv = nv;
    v.vol = vol.get(); v.cx = cx.get();
    v.cs_ptr = cs_ptr.get(); v.cs_face = cs_face.get(); v.cs_k = cs_k.get();
    v.ss_ptr = ss_ptr.get(); v.ss_w = ss_w.get(); v.ss_f = ss_f.get(); v.ss_n = ss_n.get();
    v.ss_tot = (int)ss_f.size();
    v.lsq_c = nullptr;  // Green-Gauss unless option "gradient" selects least squares
    v.fc1 = fc1.get(); v.fc2 = fc2.get();
    v.fn = fn.get(); v.farea = farea.get(); v.flam = flam.get(); v.frl = frl.get(); v.fx = fx.get();
    v.fxpac = fxpac.get(); v.fxnac = fxnac.get(); v.fd12 = fd12.get();
    v.bcell = bcell.get(); v.btype1 = btype1.get(); v.btype2 = btype2.get(); v.brid = brid.get();
    v.bdist = bdist.get(); v.bquirk_area = bquirk.get(); v.bin = bin.get(); v.bfixed = bfixed.get();
    v.cw_ptr = cw_ptr.get(); v.cw_b = cw_b.get();
    v.vx = vx.get(); v.cvert = cvert.get(); v.vc_ptr = vc_ptr.get(); v.vc_cell = vc_cell.get();
    v.A = SellView{A.n, A.nslices, A.sl_ptr.get(), A.sl_w.get(), A.col.get(), nullptr};
}

// ---------------------------------------------------------------------------
SimpleSolver::SimpleSolver(const std::string &param_path) {
    {
        size_t slash = param_path.find_last_of('/');
        case_dir = slash == std::string::npos ? "." : param_path.substr(0, slash);
    }
    cs.params = parse_params(param_path);
    std::string grid = cs.params.gridfile;
    RawMesh raw;
    try {
        raw = read_msh(grid);
    } catch (const CaseError &) {
        // the reference opens the grid relative to the working directory; also
        // accept it relative to the param file
        size_t slash = param_path.find_last_of('/');
        if (slash == std::string::npos || (!grid.empty() && grid[0] == '/')) throw;
        raw = read_msh(param_path.substr(0, slash + 1) + grid);
    }
    const Params &p = cs.params;
    if (p.density_model != 0 && p.density_model != 1) throw CaseError{"no such density model"};
    // perfect gas: the p' matrix is not symmetric (the reference switches p' to
    // GMRES, navier_pressure.cpp:28-31); the default mode runs it with BiCGSTAB
    if (p.density_model == 1) opt.p.kind = SK_BICGSTAB;
    if (p.heat_conduction && !p.solve_energy)
        throw CaseError{"must turn on SolveEnergy, if Solve3DHeatConduction is on"};
    build_case(raw, cs);
    SYSU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    fd.build(cs.fluid, cs.params, st);
    alloc_fields(f, fd, false);
    if (cs.has_solid) {
        sd.build(cs.solid, cs.params, st);
        alloc_fields(s, sd, true);
    }
    infos.alloc(SLOT_N + 3);
    infos.zero(st);
    red_blocks = 2048;
    red_partials.alloc((size_t)RED_NSLOT * red_blocks);
    red_out.alloc(RED_NSLOT);
    red_ticket.alloc(1);
    flags.alloc(1);
    flags.zero(st);
    rs = RedScratch{red_partials.get(), red_out.get(), red_ticket.get(), red_blocks};
    red_reset(rs, st);
    for (auto &e : ev) SYSU_CUDA(cudaEventCreate(&e));
    init_flow_field();
    SYSU_CUDA(cudaStreamSynchronize(st));
}

SimpleSolver::~SimpleSolver() {
    if (st) cudaStreamSynchronize(st);
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    if (st) cudaStreamDestroy(st);
}

void SimpleSolver::alloc_fields(FieldSet &fs, const DomainDev &d, bool solid) {
    size_t nc = d.nc, nf = d.nf, B = std::max(d.B, 1), F = std::max(d.F, 1), nnz = d.A.nnz;
    auto z = [&](DevBuf<double> &b, size_t n) {
        b.alloc(n);
        b.zero(st);
    };
    z(fs.T, nc); z(fs.R, nc); z(fs.dPhi, 3 * nc); z(fs.BTem, B); z(fs.Bq, B); z(fs.As, nnz);
    z(fs.bs, nc); z(fs.xs, nc); z(fs.fD, F); z(fs.fE, 3 * F); z(fs.bapp, B); z(fs.bsrc, 3 * B);
    z(fs.zeros, nc); z(fs.src, nc); z(fs.tmp3, 3 * nc); z(fs.tmpv, 2 * (size_t)std::max(d.nv, 1));
    if (!cs.params.steady) {
        z(fs.Tnp, nc);
        z(fs.tapp, nc);
    }
    if (solid) {
        z(fs.diff, nc);
        return;
    }
    if (!cs.params.steady) {
        z(fs.Unp, nc); z(fs.Vnp, nc); z(fs.Wnp, nc); z(fs.TEp, nc); z(fs.EDp, nc);
    }
    z(fs.U, nc); z(fs.V, nc); z(fs.W, nc); z(fs.P, nc); z(fs.TE, nc); z(fs.ED, nc);
    z(fs.VisLam, nc); z(fs.VisTur, nc); z(fs.Apr, nc);
    z(fs.dU, 3 * nc); z(fs.dV, 3 * nc); z(fs.dW, 3 * nc); z(fs.dP, 3 * nc);
    z(fs.RUFace, nf);
    z(fs.BRo, B); z(fs.BU, B); z(fs.BV, B); z(fs.BW, B); z(fs.BPre, B); z(fs.BTE, B); z(fs.BED, B);
    z(fs.Amom, nnz); z(fs.Ap, nnz);
    z(fs.b3, 3 * nc); z(fs.bp, nc); z(fs.x3, 3 * nc); z(fs.xp, nc);
    z(fs.fcoef, F);
    z(fs.Prod, nc); z(fs.TESrc, nc); z(fs.EDSrc, nc); z(fs.VisTE, nc); z(fs.VisED, nc);
    z(fs.ApTE, nc); z(fs.ApED, nc); z(fs.kcond, nc);
    if (cs.params.tur_model == 1 && cs.params.solve_energy) {
        z(fs.As2, nnz); z(fs.As3, nnz); z(fs.bs2, nc); z(fs.bs3, nc); z(fs.xs2, nc); z(fs.xs3, nc);
    }
}

// navier.cpp:113-188 and HeatConductionSolver.cpp:334-369
void SimpleSolver::init_flow_field() {
    const Params &p = cs.params;
    const Domain &d = cs.fluid;
    int nc = d.nc;
    std::vector<double> U(nc), V(nc), W(nc), R(nc), T(nc), P(nc, 0.0), VL(nc), VT(nc, 0.0), TE(nc, 0.0), ED(nc, 0.0);
    auto apply = [&](int i, const double *iv, size_t niv) {
        auto at = [&](size_t k) { return k < niv ? iv[k] : 0.0; };
        U[i] = at(0); V[i] = at(1); W[i] = at(2); R[i] = at(3); T[i] = at(4); P[i] = 0.0;
        if (p.density_model == 1) R[i] = (P[i] + p.pressure_reference) / (p.rcpcv() * T[i]);
        VL[i] = at(5);
        VT[i] = 0.;
        if (p.tur_model == 1) {
            TE[i] = at(6);
            ED[i] = at(7);
            VT[i] = R[i] * CMU * TE[i] * TE[i] / (ED[i] + SMALL);
        }
    };
    for (int i = 0; i < nc; ++i) {
        if (p.has_initflow) apply(i, p.initflow.data(), p.initflow.size());
        const Region &rg = p.regions.at(d.cell_rid[i]);
        apply(i, rg.initvalues, 10);
    }
    std::vector<double> BTem(std::max(d.nb, 1), 0.0), Bq(std::max(d.nb, 1), 0.0);
    for (int b = 0; b < d.nb; ++b) {
        const Region &rg = p.regions.at(d.bnd_rid[b]);
        if (rg.type1 == 1) {
            if (rg.type2 == 0) BTem[b] = rg.fixedValue;
            else if (rg.type2 == 1) Bq[b] = rg.fixedValue;
            else if (rg.type2 == 2) Bq[b] = 0.0;
        } else if (rg.type1 == 2) {
            BTem[b] = rg.initvalues[5];
        } else if (rg.type1 == 4) {
            Bq[b] = 0.0;
        }
    }
    f.U.upload(U.data(), nc, st); f.V.upload(V.data(), nc, st); f.W.upload(W.data(), nc, st);
    f.R.upload(R.data(), nc, st); f.T.upload(T.data(), nc, st); f.P.upload(P.data(), nc, st);
    f.VisLam.upload(VL.data(), nc, st); f.VisTur.upload(VT.data(), nc, st);
    f.TE.upload(TE.data(), nc, st); f.ED.upload(ED.data(), nc, st);
    f.BTem.upload(BTem.data(), d.nb, st); f.Bq.upload(Bq.data(), d.nb, st);
    f.RUFace.zero(st);
    if (cs.has_solid) {
        const Domain &sdm = cs.solid;
        int ns = sdm.nc;
        std::vector<double> Ts(ns), Rs(ns), Ks(ns);
        for (int i = 0; i < ns; ++i) {
            const Region &rg = p.regions.at(sdm.cell_rid[i]);
            Ts[i] = rg.initvalues[0];
            Rs[i] = rg.initvalues[1];
            Ks[i] = rg.initvalues[2];
        }
        std::vector<double> sB(std::max(sdm.nb, 1), 0.0), sq(std::max(sdm.nb, 1), 0.0);
        for (int b = 0; b < sdm.nb; ++b) {
            const Region &rg = p.regions.at(sdm.bnd_rid[b]);
            if (rg.type1 == 1) {
                if (rg.type2 == 0) sB[b] = rg.fixedValue;
                else if (rg.type2 == 1) sq[b] = rg.fixedValue;
                else if (rg.type2 == 2) sq[b] = 0.0;
            } else if (rg.type1 == 4) {
                sq[b] = 0.0;
            }
        }
        s.T.upload(Ts.data(), ns, st); s.R.upload(Rs.data(), ns, st); s.diff.upload(Ks.data(), ns, st);
        s.BTem.upload(sB.data(), sdm.nb, st); s.Bq.upload(sq.data(), sdm.nb, st);
        launch_bc_temperature_solid(sd.view, s.T.get(), s.diff.get(), s.Bq.get(), s.BTem.get(), st);
        const double *phi[1] = {s.T.get()};
        const double *Bphi[1] = {s.BTem.get()};
        double *grad[1] = {s.dPhi.get()};
        grad_limited(sd, s, 1, phi, Bphi, grad);
    }
}

// Option "gradient": 0 Green-Gauss (BasicSolver.cpp:29-77, the reference's), 1 least
// squares (fv.cu k_gradient_lsq) for every gradient of both domains.
void SimpleSolver::set_gradient_scheme(int scheme) {
    if (scheme != 0 && scheme != 1) throw CaseError{"gradient: 0 Green-Gauss, 1 least squares"};
    for (DomainDev *d : {&fd, &sd}) {
        if (d->nc == 0) continue;
        if (scheme == 1) {
            if (d->lsq_c.size() < (size_t)3 * d->view.ss_tot) d->lsq_c.alloc((size_t)3 * d->view.ss_tot);
            launch_lsq_setup(d->view, d->lsq_c.get(), st);
            d->view.lsq_c = d->lsq_c.get();
        } else {
            d->view.lsq_c = nullptr;
        }
    }
    gradient_scheme = scheme;
}

void SimpleSolver::grad_limited(DomainDev &d, FieldSet &fs, int nfield, const double *const *phi,
                                const double *const *Bphi, double *const *grad) {
    launch_gradient(d.view, nfield, phi, Bphi, grad, st);
    for (int k = 0; k < nfield; ++k)
        launch_limiter(d.view, cs.params.limiter, phi[k], grad[k], fs.tmp3.get(), fs.tmpv.get(), st);
}

void SimpleSolver::solve(int slot, const EqOpts &o, const SellDev &A, const double *val, int nrhs,
                         const double *const *b, double *const *x, bool x0_zero) {
    mom3.device_loop = gnn.device_loop = gnn_c.device_loop = opt.graph_loops;
    KrylovOpts ko;
    ko.maxit = o.maxit;
    ko.eps = o.eps;
    ko.omega = o.omega;
    ko.jacobi = o.precond == PK_JACOBI;
    SolveInfo *info = infos.get() + slot;
    if (nrhs == 3) mom_split = true;  // statistics per component, unless the batched form runs below
    if (o.kind == SK_GMRES) {
        // one restarted GMRES per right-hand side (the reference solves u, v, w in turn)
        for (int c = 0; c < nrhs; ++c)
            gmres_solve(A, val, b[c], x[c], x0_zero, ko, o.precond, o.restart, kw,
                        nrhs == 1 ? info : infos.get() + SLOT_N + c, st);
        return;
    }
    if (o.kind == SK_CG && (o.learned || o.precond == PK_AMG) && &A == &fd.A) {
        if (nrhs != 1) throw CaseError{"CG solves one right-hand side"};
        solve_learned(o, val, b[0], x[0], x0_zero, info);
        return;
    }
    if (o.kind == SK_CG) {
        if (nrhs != 1) throw CaseError{"CG solves one right-hand side"};
        if (o.precond == PK_SSOR || o.precond == PK_ILU0) {
            pcg_solve(A, val, b[0], x[0], x0_zero, ko, o.precond, kw, info, st);
            return;
        }
        if (o.mixed) {
            // FP32 copy of this equation's matrix, then FP32 inner / FP64 outer CG
            DevBuf<float> &v32 = (&A == &sd.A) ? s.As32 : f.Ap32;
            if (v32.size() < (size_t)A.nnz) v32.alloc(A.nnz);
            sell_to_fp32(A, val, v32.get(), st);
            ko.inner_tol = o.inner_tol;
            cg_solve_mixed(A, val, v32.get(), b[0], x[0], x0_zero, ko, kw, info, st);
            return;
        }
        cg_solve(A, val, b[0], x[0], x0_zero, ko, kw, info, st);
        return;
    }
    if (x0_zero)
        for (int c = 0; c < nrhs; ++c) launch_fill(x[c], 0.0, A.n, st);
    if (o.mixed) {
        ko.inner_tol = o.inner_tol;
        if (nrhs == 1) {
            bicgstab_solve_mixed(A, val, b[0], x[0], ko, kw, info, st);
            return;
        }
        if (nrhs == 3 && opt.mom_batched) {
            // momentum: u, v, w together, FP32 recurrences with FP64 residual
            // replacement (graph-resident: also inside a captured outer iteration)
            mom3.solve(A, val, b, x, ko, kw, info, st);
            mom_split = false;
            return;
        }
        // momentum unbatched: u, v, w one after another, each a persistent solve
        // with FP32 inner iterations in FP64 defect correction (statistics per
        // component)
        for (int c = 0; c < nrhs; ++c) bicgstab_solve_mixed(A, val, b[c], x[c], ko, kw, infos.get() + SLOT_N + c, st);
        return;
    }
    if (nrhs == 3 && !opt.mom_batched) {
        for (int c = 0; c < 3; ++c) bicgstab_solve(A, val, 1, &b[c], &x[c], ko, kw, infos.get() + SLOT_N + c, st);
        return;
    }
    if (nrhs == 3) mom_split = false;
    bicgstab_solve(A, val, nrhs, b, x, ko, kw, info, st);
}

// p' solve of the learned and multigrid forms.  With precond PK_AMG the
// flexible CG is preconditioned by the aggregation-multigrid cycle (hierarchy
// built at the first solve, values refreshed at every solve); with learned set,
// the network is that cycle's finest post-smoother (without PK_AMG: the whole
// preconditioner).  Training window of the learned form: a loose plain solve
// (1e-2) from zero, then the solve to eps from there; the pairs (b, x*) and
// (b - A x1, x* - x1) go into the network's ring (as post-smoother pairs in the
// multigrid form) and learn_steps Adam steps follow.  After the window: flexible
// CG with the network.
void SimpleSolver::solve_learned(const EqOpts &o, const double *val, const double *b, double *x, bool x0_zero,
                                 SolveInfo *info) {
    const SellDev &A = fd.A;
    const bool use_mg = o.precond == PK_AMG;
    if (f.Ap32.size() < (size_t)A.nnz) f.Ap32.alloc(A.nnz);
    sell_to_fp32(A, val, f.Ap32.get(), st);
    if (!gnn.bound()) {
        gnn.set_capacity(std::max(8, 2 * std::min(o.learn_iters, 32)));
        gnn.bind(A, val, f.Ap32.get(), st);
        gnn.init_params(20261203ULL, st);
        gnn.loss_kind = o.learn_kind;
    } else {
        gnn.refresh(st);
    }
    int lvl = 0;  // level of the network in the multigrid form
    if (use_mg) {
        if (!mg.ready() || mg_theta_built != o.mg_theta) {
            gnn.attach_multigrid(nullptr);
            mg.setup(A, fd.pat, val, o.mg_theta, st);
            mg_theta_built = o.mg_theta;
            learn_level_built = -1;
        }
        mg.omega = o.mg_omega;
        mg.gamma = o.mg_gamma;
        mg.persistent = o.mg_persistent != 0;  // part of the captured iterations' key
        mg.refresh(val, f.Ap32.get(), st);
        if (o.learned) lvl = std::max(0, std::min(o.learn_level, mg.levels() - 2));
        if (lvl >= 1) {
            if (learn_level_built != lvl) {
                gnn.attach_multigrid(nullptr);  // the captured iterations change
                gnn_c.set_capacity(std::max(8, 2 * std::min(o.learn_iters, 32)));
                gnn_c.bind(mg.level_matrix(lvl), mg.level_val64(lvl), mg.level_val32(lvl), st);
                gnn_c.init_params(20261203ULL, st);
                mg_c.omega = o.mg_omega;
                mg_c.gamma = o.mg_gamma;
                mg_c.setup(mg.level_matrix(lvl), mg.level_pattern(lvl), mg.level_val64(lvl), o.mg_theta, st);
                learn_level_built = lvl;
            }
            gnn_c.loss_kind = o.learn_kind;
            gnn_c.skip = (float)o.mg_omega;
            if (p_solves < o.learn_iters) {
                // the level's own hierarchy serves the training pairs' level solves only
                mg_c.omega = o.mg_omega;
                mg_c.gamma = o.mg_gamma;
                mg_c.refresh(mg.level_val64(lvl), mg.level_val32(lvl), st);
            }
            gnn_c.refresh(st);
            if (gnn_c.multigrid() != &mg_c) gnn_c.attach_multigrid(&mg_c);
            mg.post_level = lvl;
            mg.post_hook = [this](int l, const float *r, const float *zp, float *z, const int *, cudaStream_t s) {
                gnn_c.post_smooth(r, zp, z, gnn.fcg_state(), mg.level_w(l), s);
            };
        } else {
            mg.post_level = -1;
            mg.post_hook = nullptr;
        }
        gnn.net_level = lvl;
        gnn.skip = (float)o.mg_omega;  // the finest-level network as the cycle's post-smoother
        if (gnn.multigrid() != &mg) gnn.attach_multigrid(&mg);
    } else {
        if (gnn.multigrid()) gnn.attach_multigrid(nullptr);
        gnn.net_level = 0;
        gnn.skip = 1.0f;  // the network as the whole preconditioner
    }
    KrylovOpts ko;
    ko.maxit = o.maxit;
    ko.eps = o.eps;
    ko.omega = o.omega;
    ko.jacobi = true;
    ko.inner_tol = o.inner_tol;
    // the multigrid's error flag (a bounded wait timed out, the coarsest level is
    // singular) is read with the outer iteration's other results (check_iteration)
    if (!o.learned) {
        gnn.fcg(b, x, x0_zero, ko, false, info, st);
        return;
    }
    if (stream_capturing(st)) throw CaseError{"the learned p' form trains on the host's schedule: not in a captured graph"};
    if (p_solves++ >= o.learn_iters) {
        gnn.fcg(b, x, x0_zero, ko, true, info, st);
        return;
    }
    auto plain = [&](double eps, bool zero) {
        KrylovOpts k = ko;
        k.eps = eps;
        if (use_mg) gnn.fcg(b, x, zero, k, false, info, st);
        else if (o.mixed) cg_solve_mixed(A, val, f.Ap32.get(), b, x, zero, k, kw, info, st);
        else cg_solve(A, val, b, x, zero, k, kw, info, st);
    };
    if (gnn_x1.size() < (size_t)A.n) gnn_x1.alloc(A.n);
    plain(std::max(o.eps, 1e-2), x0_zero);
    SYSU_CUDA(cudaMemcpyAsync(gnn_x1.get(), x, sizeof(double) * A.n, cudaMemcpyDeviceToDevice, st));
    plain(o.eps, false);
    if (lvl >= 1) {
        // pairs of the coarse level: the right-hand side the cycle hands that level
        // for the finest residuals b and b - A x1, and the level's own solution of
        // it (flexible CG with the hierarchy below the level); add_pair turns them
        // into post-smoother pairs of that level
        const int nl = mg.level_rows(lvl);
        if (mg_r32.size() < (size_t)A.n) mg_r32.alloc(A.n);
        if (mg_rl32.size() < (size_t)nl) {
            mg_rl32.alloc(nl);
            mg_rl64.alloc(nl);
            mg_el64.alloc(nl);
        }
        if (!mg_info.size()) mg_info.alloc(1);
        KrylovOpts kl = ko;
        kl.eps = 1e-6;
        kl.maxit = 1000;
        for (const double *x1 : {static_cast<const double *>(nullptr), static_cast<const double *>(gnn_x1.get())}) {
            gnn.residual32(b, x1, mg_r32.get(), st);
            mg.level_rhs(lvl, mg_r32.get(), mg_rl32.get(), st);
            mg_to_f64(mg_rl32.get(), mg_rl64.get(), nl, st);
            gnn_c.fcg(mg_rl64.get(), mg_el64.get(), true, kl, false, mg_info.get(), st);
            gnn_c.add_pair(mg_rl64.get(), mg_el64.get(), st);
        }
        for (int k = 0; k < o.learn_steps; ++k) gnn_c.train_step(k % gnn_c.pairs(), o.learn_lr, st);
        return;
    }
    gnn.add_pair_from(b, nullptr, x, st);
    gnn.add_pair_from(b, gnn_x1.get(), x, st);
    for (int k = 0; k < o.learn_steps; ++k) gnn.train_step(k % gnn.pairs(), o.learn_lr, st);
}

void SimpleSolver::p_cycle(const double *r, double *z, bool use_net) {
    if (!mg.ready() || gnn.multigrid() != &mg) throw CaseError{"p' multigrid: no p' solve with precond 4 yet"};
    const int n = fd.A.n;
    if (mg_r32.size() < (size_t)n) mg_r32.alloc(n);
    DevBuf<double> d(n);
    DevBuf<float> z32(n);
    d.upload(r, n, st);
    gnn.residual32(d.get(), nullptr, mg_r32.get(), st);
    // the cycle's network kernels read the flexible CG's flags: running, network on or off
    FcgState *fs = gnn.fcg_state();
    const int flags[2] = {0, use_net ? 1 : 0};
    SYSU_CUDA(cudaMemcpyAsync(&fs->done, &flags[0], sizeof(int), cudaMemcpyHostToDevice, st));
    SYSU_CUDA(cudaMemcpyAsync(&fs->use_gnn, &flags[1], sizeof(int), cudaMemcpyHostToDevice, st));
    if (gnn.net_level == 0 && use_net) {
        gnn.apply_mg(d.get(), d.get(), true, st);
    } else {
        mg.apply(mg_r32.get(), z32.get(), &fs->done, st);
        mg_to_f64(z32.get(), d.get(), n, st);
    }
    d.download(z, n, st);
    SYSU_CUDA(cudaStreamSynchronize(st));
}

// CalculateVelocity + BuildVelocityMatrix, navier_velocity.cpp:12-357
void SimpleSolver::calculate_velocity() {
    const Params &p = cs.params;
    const DomView &d = fd.view;
    int nc = fd.nc;
    launch_bc_velocity(d, f.R.get(), f.U.get(), f.V.get(), f.W.get(), f.BRo.get(), f.BU.get(), f.BV.get(),
                       f.BW.get(), fd.has_outlet && p.density_model == 0, rs, st);
    launch_bnd_from_cell(d, f.P.get(), f.BPre.get(), st);
    const double *phi[4] = {f.U.get(), f.V.get(), f.W.get(), f.P.get()};
    const double *Bphi[4] = {f.BU.get(), f.BV.get(), f.BW.get(), f.BPre.get()};
    double *grad[4] = {f.dU.get(), f.dV.get(), f.dW.get(), f.dP.get()};
    grad_limited(fd, f, 4, phi, Bphi, grad);
    MomArgs a{};
    a.U = f.U.get(); a.V = f.V.get(); a.W = f.W.get(); a.R = f.R.get();
    a.VisLam = f.VisLam.get(); a.VisTur = f.VisTur.get(); a.RUFace = f.RUFace.get();
    a.dU = f.dU.get(); a.dV = f.dV.get(); a.dW = f.dW.get(); a.dP = f.dP.get();
    a.BU = f.BU.get(); a.BV = f.BV.get(); a.BW = f.BW.get();
    a.urf = p.urf[0];
    for (int k = 0; k < 3; ++k) a.g[k] = p.gravity[k];
    a.fD = f.fD.get(); a.fE = f.fE.get(); a.bapp = f.bapp.get(); a.bsrc = f.bsrc.get();
    a.val = f.Amom.get();
    a.tscheme = tscheme();
    a.hybrid = opt.convection == 1;
    if (a.tscheme) {
        a.Unp = f.Unp.get(); a.Vnp = f.Vnp.get(); a.Wnp = f.Wnp.get();
        a.dt = p.dt;
    }
    a.bu = f.b3.get(); a.bv = f.b3.get() + nc; a.bw = f.b3.get() + 2 * (size_t)nc;
    a.Apr = f.Apr.get();
    a.flags = flags.get();
    launch_momentum(d, a, st);
    launch_copy(f.x3.get(), f.U.get(), nc, st);
    launch_copy(f.x3.get() + nc, f.V.get(), nc, st);
    launch_copy(f.x3.get() + 2 * (size_t)nc, f.W.get(), nc, st);
    const double *b[3] = {a.bu, a.bv, a.bw};
    double *x[3] = {f.x3.get(), f.x3.get() + nc, f.x3.get() + 2 * (size_t)nc};
    if (opt.timing) SYSU_CUDA(cudaEventRecord(ev[2], st));
    solve(SLOT_MOM, opt.mom, fd.A, f.Amom.get(), 3, b, x, false);
    if (opt.timing) SYSU_CUDA(cudaEventRecord(ev[3], st));
    launch_commit3(d, f.U.get(), f.V.get(), f.W.get(), f.x3.get(), rs, st);
}

// CalculatePressure, navier_pressure.cpp:9-76
void SimpleSolver::calculate_pressure() {
    const Params &p = cs.params;
    const DomView &d = fd.view;
    launch_bc_velocity(d, f.R.get(), f.U.get(), f.V.get(), f.W.get(), f.BRo.get(), f.BU.get(), f.BV.get(),
                       f.BW.get(), fd.has_outlet && p.density_model == 0, rs, st);
    PresArgs pa{};
    pa.U = f.U.get(); pa.V = f.V.get(); pa.W = f.W.get(); pa.R = f.R.get(); pa.P = f.P.get();
    pa.dP = f.dP.get(); pa.Apr = f.Apr.get();
    pa.BRo = f.BRo.get(); pa.BU = f.BU.get(); pa.BV = f.BV.get(); pa.BW = f.BW.get();
    pa.RUFace = f.RUFace.get(); pa.fcoef = f.fcoef.get(); pa.val = f.Ap.get(); pa.bp = f.bp.get();
    pa.density_model = p.density_model; pa.T = f.T.get(); pa.rcpcv = p.rcpcv();
    pa.transient = tscheme() != 0; pa.dt = p.dt;
    launch_pressure_assembly(d, pa, st);
    const double *b[1] = {f.bp.get()};
    double *x[1] = {f.xp.get()};
    if (opt.timing) SYSU_CUDA(cudaEventRecord(ev[0], st));
    solve(SLOT_P, opt.p, fd.A, f.Ap.get(), 1, b, x, true);
    if (opt.timing) SYSU_CUDA(cudaEventRecord(ev[1], st));
    launch_bnd_from_cell(d, f.xp.get(), f.BPre.get(), st);
    const double *phi[1] = {f.xp.get()};
    const double *Bphi[1] = {f.BPre.get()};
    double *grad[1] = {f.dP.get()};
    grad_limited(fd, f, 1, phi, Bphi, grad);
    CorrArgs ca{};
    ca.dp = f.xp.get(); ca.dPdp = f.dP.get(); ca.Apr = f.Apr.get(); ca.R = f.R.get();
    ca.P = f.P.get(); ca.U = f.U.get(); ca.V = f.V.get(); ca.W = f.W.get();
    ca.urf_p = p.urf[3];
    ca.cell_ref = p.cell_pressure_ref;
    ca.density_model = p.density_model; ca.T = f.T.get(); ca.rcpcv = p.rcpcv();
    launch_correct_cells(d, ca, rs, st);
    launch_bc_velocity(d, f.R.get(), f.U.get(), f.V.get(), f.W.get(), f.BRo.get(), f.BU.get(), f.BV.get(),
                       f.BW.get(), fd.has_outlet && p.density_model == 0, rs, st);
    launch_correct_faces(d, f.xp.get(), f.dP.get(), f.R.get(), f.Apr.get(), f.BRo.get(), f.BU.get(), f.BV.get(),
                         f.BW.get(), p.urf[3], f.RUFace.get(), f.fcoef.get(), p.density_model, f.T.get(), p.rcpcv(),
                         st);
}

// UpdateTurKEpsilon, navier_scalar.cpp:14-172
void SimpleSolver::update_ke() {
    const Params &p = cs.params;
    const DomView &d = fd.view;
    int nc = fd.nc;
    KeArgs k{};
    k.dU = f.dU.get(); k.dV = f.dV.get(); k.dW = f.dW.get(); k.R = f.R.get(); k.VisLam = f.VisLam.get();
    k.U = f.U.get(); k.V = f.V.get(); k.W = f.W.get();
    k.TE = f.TE.get(); k.ED = f.ED.get(); k.VisTur = f.VisTur.get();
    k.Prod = f.Prod.get(); k.TESrc = f.TESrc.get(); k.EDSrc = f.EDSrc.get(); k.VisTE = f.VisTE.get();
    k.VisED = f.VisED.get(); k.ApTE = f.ApTE.get(); k.ApED = f.ApED.get(); k.BTE = f.BTE.get(); k.BED = f.BED.get();
    launch_ke_sources(d, k, st);
    launch_ke_bnd_values(d, k, st);
    // unsteady terms after the boundary treatment (navier_scalar.cpp:72-89); the
    // eps source is recomputed after the k solve, so only its diagonal keeps it
    launch_time_term(nc, f.R.get(), fd.vol.get(), p.dt, tscheme(), f.TEp.get(), f.ApTE.get(), f.TESrc.get(), st);
    launch_time_term(nc, f.R.get(), fd.vol.get(), p.dt, tscheme(), f.EDp.get(), f.ApED.get(), f.EDSrc.get(), st);
    ScalarArgs sa{};
    sa.hybrid = opt.convection == 1;
    sa.RUFace = f.RUFace.get(); sa.grad = f.dPhi.get(); sa.urf = p.urf[5]; sa.bc_mode = SC_FLUID_PLAIN;
    sa.fD = f.fD.get(); sa.fE = f.fE.get(); sa.bapp = f.bapp.get(); sa.bsrc = f.bsrc.get();
    sa.val = f.As.get(); sa.b = f.bs.get(); sa.flags = flags.get();
    {
        const double *phi[1] = {f.TE.get()};
        const double *Bphi[1] = {f.BTE.get()};
        double *grad[1] = {f.dPhi.get()};
        grad_limited(fd, f, 1, phi, Bphi, grad);
        sa.phi = f.TE.get(); sa.Bphi = f.BTE.get(); sa.diff = f.VisTE.get(); sa.src = f.TESrc.get(); sa.app0 = f.ApTE.get();
        launch_scalar(d, sa, st);
        launch_copy(f.xs.get(), f.TE.get(), nc, st);
        const double *b[1] = {f.bs.get()};
        double *x[1] = {f.xs.get()};
        solve(SLOT_K, opt.ke, fd.A, f.As.get(), 1, b, x, false);
        launch_clip_max(f.TE.get(), f.xs.get(), 1.e-9, nc, st);
    }
    launch_ke_eps_sources(d, k, st);
    {
        const double *phi[1] = {f.ED.get()};
        const double *Bphi[1] = {f.BED.get()};
        double *grad[1] = {f.dPhi.get()};
        grad_limited(fd, f, 1, phi, Bphi, grad);
        sa.phi = f.ED.get(); sa.Bphi = f.BED.get(); sa.diff = f.VisED.get(); sa.src = f.EDSrc.get(); sa.app0 = f.ApED.get();
        launch_scalar(d, sa, st);
        launch_ke_eps_wall_rows(d, f.ED.get(), f.As.get(), f.bs.get(), st);
        launch_copy(f.xs.get(), f.ED.get(), nc, st);
        const double *b[1] = {f.bs.get()};
        double *x[1] = {f.xs.get()};
        solve(SLOT_EPS, opt.ke, fd.A, f.As.get(), 1, b, x, false);
        launch_clip_max(f.ED.get(), f.xs.get(), 1.e-12, nc, st);
    }
    launch_visc_tur(nc, f.R.get(), f.TE.get(), f.ED.get(), f.VisTur.get(), st);
}

// Batched scalar form: UpdateTurKEpsilon and UpdateEnergy (navier_scalar.cpp:14-172,
// 257-397) assembled from the fields as they stand after the pressure
// correction, then one three-system BiCGSTAB launch.  Differences from the
// sequential form: eps's production/dissipation terms use k of the previous
// outer iteration (the reference recomputes them after the k solve) and T's
// conductivity uses the previous mu_t; a steady solution satisfies both forms.
void SimpleSolver::update_scalars_batched() {
    const Params &p = cs.params;
    const DomView &d = fd.view;
    int nc = fd.nc;
    KeArgs k{};
    k.dU = f.dU.get(); k.dV = f.dV.get(); k.dW = f.dW.get(); k.R = f.R.get(); k.VisLam = f.VisLam.get();
    k.U = f.U.get(); k.V = f.V.get(); k.W = f.W.get();
    k.TE = f.TE.get(); k.ED = f.ED.get(); k.VisTur = f.VisTur.get();
    k.Prod = f.Prod.get(); k.TESrc = f.TESrc.get(); k.EDSrc = f.EDSrc.get(); k.VisTE = f.VisTE.get();
    k.VisED = f.VisED.get(); k.ApTE = f.ApTE.get(); k.ApED = f.ApED.get(); k.BTE = f.BTE.get(); k.BED = f.BED.get();
    launch_ke_sources(d, k, st);
    launch_ke_bnd_values(d, k, st);
    launch_time_term(nc, f.R.get(), fd.vol.get(), p.dt, tscheme(), f.TEp.get(), f.ApTE.get(), f.TESrc.get(), st);
    launch_time_term(nc, f.R.get(), fd.vol.get(), p.dt, tscheme(), f.EDp.get(), f.ApED.get(), f.EDSrc.get(), st);
    launch_ke_eps_sources(d, k, st);
    ScalarArgs sa{};
    sa.hybrid = opt.convection == 1;
    sa.RUFace = f.RUFace.get(); sa.grad = f.dPhi.get(); sa.urf = p.urf[5]; sa.bc_mode = SC_FLUID_PLAIN;
    sa.fD = f.fD.get(); sa.fE = f.fE.get(); sa.bapp = f.bapp.get(); sa.bsrc = f.bsrc.get();
    sa.flags = flags.get();
    {
        const double *phi[1] = {f.TE.get()};
        const double *Bphi[1] = {f.BTE.get()};
        double *grad[1] = {f.dPhi.get()};
        grad_limited(fd, f, 1, phi, Bphi, grad);
        sa.phi = f.TE.get(); sa.Bphi = f.BTE.get(); sa.diff = f.VisTE.get(); sa.src = f.TESrc.get(); sa.app0 = f.ApTE.get();
        sa.val = f.As.get(); sa.b = f.bs.get();
        launch_scalar(d, sa, st);
        launch_copy(f.xs.get(), f.TE.get(), nc, st);
    }
    {
        const double *phi[1] = {f.ED.get()};
        const double *Bphi[1] = {f.BED.get()};
        double *grad[1] = {f.dPhi.get()};
        grad_limited(fd, f, 1, phi, Bphi, grad);
        sa.phi = f.ED.get(); sa.Bphi = f.BED.get(); sa.diff = f.VisED.get(); sa.src = f.EDSrc.get(); sa.app0 = f.ApED.get();
        sa.val = f.As2.get(); sa.b = f.bs2.get();
        launch_scalar(d, sa, st);
        launch_ke_eps_wall_rows(d, f.ED.get(), f.As2.get(), f.bs2.get(), st);
        launch_copy(f.xs2.get(), f.ED.get(), nc, st);
    }
    launch_kcond(nc, f.VisLam.get(), f.VisTur.get(), p.cp, p.prl, p.prte, f.kcond.get(), st);
    launch_bc_temperature_fluid(d, f.T.get(), f.BTem.get(), st);
    if (cs.has_solid) launch_cht_solid2fluid(sd.view, s.T.get(), s.dPhi.get(), d, f.BTem.get(), st);
    {
        const double *phi[1] = {f.T.get()};
        const double *Bphi[1] = {f.BTem.get()};
        double *grad[1] = {f.dPhi.get()};
        grad_limited(fd, f, 1, phi, Bphi, grad);
        ScalarArgs ta = sa;
        ta.phi = f.T.get(); ta.Bphi = f.BTem.get(); ta.diff = f.kcond.get(); ta.src = f.zeros.get(); ta.app0 = f.zeros.get();
        energy_sources(ta);
        ta.Bq = f.Bq.get();
        ta.bc_mode = SC_FLUID_ENERGY;
        ta.val = f.As3.get(); ta.b = f.bs3.get();
        launch_scalar(d, ta, st);
        launch_copy(f.xs3.get(), f.T.get(), nc, st);
    }
    KrylovOpts ko;
    ko.maxit = opt.ke.maxit;
    ko.eps = opt.ke.eps;
    ko.omega = opt.ke.omega;
    ko.jacobi = opt.ke.precond == PK_JACOBI;
    const double *vals[3] = {f.As.get(), f.As2.get(), f.As3.get()};
    const double *bb[3] = {f.bs.get(), f.bs2.get(), f.bs3.get()};
    double *xx[3] = {f.xs.get(), f.xs2.get(), f.xs3.get()};
    bicgstab_solve_multi(fd.A, vals, bb, xx, ko, kw, infos.get() + SLOT_K, st);
    launch_clip_max(f.TE.get(), f.xs.get(), 1.e-9, nc, st);
    launch_clip_max(f.ED.get(), f.xs2.get(), 1.e-12, nc, st);
    launch_visc_tur(nc, f.R.get(), f.TE.get(), f.ED.get(), f.VisTur.get(), st);
    launch_copy(f.T.get(), f.xs3.get(), nc, st);
    if (cs.has_solid)
        launch_cht_fluid2solid(d, f.dPhi.get(), f.kcond.get(), f.Bq.get(), sd.view, s.Bq.get(), st);
}

// Source and extra diagonal of the fluid energy equation: the viscous work of
// density model 1 (navier_scalar.cpp:277-338) and the unsteady term
// (navier_scalar.cpp:350-366), in the reference's order.
void SimpleSolver::energy_sources(ScalarArgs &sa) {
    const Params &p = cs.params;
    int nc = fd.nc;
    if (!tscheme() && p.density_model != 1) return;
    launch_fill(f.src.get(), 0.0, nc, st);
    sa.src = f.src.get();
    if (p.density_model == 1)
        launch_energy_viscous(fd.view, f.VisLam.get(), f.VisTur.get(), f.dU.get(), f.dV.get(), f.dW.get(), f.U.get(),
                              f.V.get(), f.W.get(), p.cp, f.src.get(), st);
    if (tscheme()) {
        launch_fill(f.tapp.get(), 0.0, nc, st);
        launch_time_term(nc, f.R.get(), fd.vol.get(), p.dt, tscheme(), f.Tnp.get(), f.tapp.get(), f.src.get(), st);
        sa.app0 = f.tapp.get();
    }
}

// NavierStokesSolver::UpdateEnergy, navier_scalar.cpp:257-397
void SimpleSolver::update_energy() {
    const Params &p = cs.params;
    const DomView &d = fd.view;
    int nc = fd.nc;
    launch_kcond(nc, f.VisLam.get(), f.VisTur.get(), p.cp, p.prl, p.prte, f.kcond.get(), st);
    launch_bc_temperature_fluid(d, f.T.get(), f.BTem.get(), st);
    if (cs.has_solid) launch_cht_solid2fluid(sd.view, s.T.get(), s.dPhi.get(), d, f.BTem.get(), st);
    const double *phi[1] = {f.T.get()};
    const double *Bphi[1] = {f.BTem.get()};
    double *grad[1] = {f.dPhi.get()};
    grad_limited(fd, f, 1, phi, Bphi, grad);
    ScalarArgs sa{};
    sa.hybrid = opt.convection == 1;
    sa.phi = f.T.get(); sa.Bphi = f.BTem.get(); sa.diff = f.kcond.get(); sa.src = f.zeros.get(); sa.app0 = f.zeros.get();
    energy_sources(sa);
    sa.grad = f.dPhi.get(); sa.RUFace = f.RUFace.get(); sa.Bq = f.Bq.get(); sa.urf = p.urf[5];
    sa.bc_mode = SC_FLUID_ENERGY;
    sa.fD = f.fD.get(); sa.fE = f.fE.get(); sa.bapp = f.bapp.get(); sa.bsrc = f.bsrc.get();
    sa.val = f.As.get(); sa.b = f.bs.get(); sa.flags = flags.get();
    launch_scalar(d, sa, st);
    launch_copy(f.xs.get(), f.T.get(), nc, st);
    const double *b[1] = {f.bs.get()};
    double *x[1] = {f.xs.get()};
    solve(SLOT_T, opt.t, fd.A, f.As.get(), 1, b, x, false);
    launch_copy(f.T.get(), f.xs.get(), nc, st);
    if (cs.has_solid)
        launch_cht_fluid2solid(d, f.dPhi.get(), f.kcond.get(), f.Bq.get(), sd.view, s.Bq.get(), st);
}

// HeatConductionSolver::UpdateEnergy, HeatConductionSolver.cpp:47-106
void SimpleSolver::solid_solve() {
    const DomView &d = sd.view;
    int nc = sd.nc;
    if (opt.solid_source != 0.0) launch_scale_src(s.src.get(), sd.vol.get(), opt.solid_source, nc, st);
    else launch_fill(s.src.get(), 0.0, nc, st);
    launch_bc_temperature_solid(d, s.T.get(), s.diff.get(), s.Bq.get(), s.BTem.get(), st);
    const double *phi[1] = {s.T.get()};
    const double *Bphi[1] = {s.BTem.get()};
    double *grad[1] = {s.dPhi.get()};
    grad_limited(sd, s, 1, phi, Bphi, grad);
    ScalarArgs sa{};
    sa.hybrid = opt.convection == 1;
    sa.phi = s.T.get(); sa.Bphi = s.BTem.get(); sa.diff = s.diff.get(); sa.src = s.src.get(); sa.app0 = s.zeros.get();
    if (tscheme()) {  // HeatConductionSolver.cpp:66-80 (solid density)
        // Always Euler: NavierStokesSolver declares its own TimeScheme (navier.h:29),
        // so the copy that seeds the solid (Preprocessor.cpp:466-468) carries the
        // base-class default 1 (BasicSolver.cpp:10) while IfSteady and dt come
        // across; a "Dual" case steps the solid with the Euler term.
        launch_fill(s.tapp.get(), 0.0, nc, st);
        launch_time_term(nc, s.R.get(), sd.vol.get(), cs.params.dt, 1, s.Tnp.get(), s.tapp.get(),
                         s.src.get(), st);
        sa.app0 = s.tapp.get();
    }
    sa.grad = s.dPhi.get(); sa.RUFace = nullptr; sa.Bq = s.Bq.get(); sa.urf = 1.0;  // Preprocessor.cpp:506
    sa.bc_mode = SC_SOLID;
    sa.fD = s.fD.get(); sa.fE = s.fE.get(); sa.bapp = s.bapp.get(); sa.bsrc = s.bsrc.get();
    sa.val = s.As.get(); sa.b = s.bs.get(); sa.flags = flags.get();
    launch_scalar(d, sa, st);
    launch_copy(s.xs.get(), s.T.get(), nc, st);
    const double *b[1] = {s.bs.get()};
    double *x[1] = {s.xs.get()};
    solve(SLOT_TS, opt.ts, sd.A, s.As.get(), 1, b, x, false);
    launch_copy(s.T.get(), s.xs.get(), nc, st);
}

void SimpleSolver::save_transient_old_data() {
    if (!tscheme()) return;
    int nc = fd.nc;
    launch_copy(f.Unp.get(), f.U.get(), nc, st);
    launch_copy(f.Vnp.get(), f.V.get(), nc, st);
    launch_copy(f.Wnp.get(), f.W.get(), nc, st);
    launch_copy(f.Tnp.get(), f.T.get(), nc, st);
    launch_copy(f.TEp.get(), f.TE.get(), nc, st);
    launch_copy(f.EDp.get(), f.ED.get(), nc, st);
    if (cs.has_solid) launch_copy(s.Tnp.get(), s.T.get(), sd.nc, st);
}

std::string SimpleSolver::outer_iteration() {
    enqueue_iteration();
    ++iter_done;
    return check_iteration();
}

void SimpleSolver::enqueue_iteration() {
    SYSU_CUDA(cudaMemsetAsync(infos.get(), 0, sizeof(SolveInfo) * (SLOT_N + 3), st));
    calculate_velocity();
    calculate_pressure();
    if (opt.scalars_batched && cs.params.tur_model == 1 && cs.params.solve_energy) {
        update_scalars_batched();
        if (cs.has_solid) solid_solve();
    } else {
        if (cs.params.tur_model == 1) update_ke();
        if (cs.params.solve_energy) {
            update_energy();
            if (cs.has_solid) solid_solve();
        }
    }
}

std::string SimpleSolver::check_iteration() {
    SolveInfo h[SLOT_N + 3];
    double ro[RED_NSLOT];
    int hf = 0;
    int mgerr = 0;
    infos.download(h, SLOT_N + 3, st);
    red_out.download(ro, RED_NSLOT, st);
    flags.download(&hf, 1, st);
    if (mg.ready()) SYSU_CUDA(cudaMemcpyAsync(&mgerr, mg.err_dev(), sizeof(int), cudaMemcpyDeviceToHost, st));
    SYSU_CUDA(cudaStreamSynchronize(st));
    if (mgerr) throw CaseError{"p' multigrid: a bounded wait timed out or the coarsest level is singular"};
    if (mom_split)
        for (int c = 0; c < 3; ++c) {
            h[SLOT_MOM].status[c] = h[SLOT_N + c].status[0];
            h[SLOT_MOM].iters[c] = h[SLOT_N + c].iters[0];
            h[SLOT_MOM].res[c] = h[SLOT_N + c].res[0];
            h[SLOT_MOM].err |= h[SLOT_N + c].err;
        }
    if (opt.scalars_batched && cs.params.tur_model == 1 && cs.params.solve_energy) {
        // one batched solve: k, eps, T in the slots of SLOT_K
        int sl[3] = {SLOT_K, SLOT_EPS, SLOT_T};
        SolveInfo b = h[SLOT_K];
        for (int c = 0; c < 3; ++c) {
            h[sl[c]] = SolveInfo{};
            h[sl[c]].status[0] = b.status[c];
            h[sl[c]].iters[0] = b.iters[c];
            h[sl[c]].res[0] = b.res[c];
            h[sl[c]].err = b.err;
        }
    }
    std::memcpy(last_info, h, sizeof(last_info));
    for (int k = 0; k < 10; ++k) Residual[k] = 0.0;
    Residual[0] = ro[RED_RES0];
    Residual[1] = ro[RED_RES1];
    Residual[2] = ro[RED_RES2];
    Residual[3] = ro[RED_RES3];
    if (opt.timing) {
        float ms = 0.f;
        SYSU_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        last_p_ms = ms;
        SYSU_CUDA(cudaEventElapsedTime(&ms, ev[2], ev[3]));
        last_mom_ms = ms;
    }
    if (hf & 1) return "no such boundary type";
    if (hf & 2) return "reverse flow get out of inlet. stop!";
    for (int k = 0; k < SLOT_N; ++k)
        if (h[k].err) return "Krylov solve aborted: a grid barrier wait timed out";
    if (!opt.fatal_checks) return "";
    static const char *names[3] = {"U", "V", "W"};
    for (int c = 0; c < 3; ++c) {
        if (h[SLOT_MOM].status[c] == DEV_NONFINITE) return std::string(names[c]) + " solve produced a non-finite residual";
        if (h[SLOT_MOM].iters[c] >= 500 && h[SLOT_MOM].res[c] > 1.e-8)  // navier_velocity.cpp:29,42,54
            return std::string(names[c]) + " cannot converge, res: : " + std::to_string(h[SLOT_MOM].res[c]);
    }
    if (!(h[SLOT_P].res[0] <= 1.))  // navier_pressure.cpp:32-34
        return "Pressure iteration cannot onverge, res: : " + std::to_string(h[SLOT_P].res[0]);
    int slots[4] = {SLOT_K, SLOT_EPS, SLOT_T, SLOT_TS};
    for (int k : slots)
        if (h[k].iters[0] >= 500 && h[k].res[0] > 1.e-8) return "Energy cannot converge.";  // navier_scalar.cpp:102-105
    return "";
}

void SimpleSolver::sync() { SYSU_CUDA(cudaStreamSynchronize(st)); }

void SimpleSolver::reset() {
    sync();
    for (double &r : Residual) r = 0.0;
    iter_done = 0;
    std::memset(last_info, 0, sizeof(last_info));
    flags.zero(st);
    red_reset(rs, st);
    init_flow_field();
    sync();
}

void SimpleSolver::timer_start() { SYSU_CUDA(cudaEventRecord(ev[4], st)); }

double SimpleSolver::timer_stop() {
    SYSU_CUDA(cudaEventRecord(ev[5], st));
    SYSU_CUDA(cudaEventSynchronize(ev[5]));
    float ms = 0.f;
    SYSU_CUDA(cudaEventElapsedTime(&ms, ev[4], ev[5]));
    return ms;
}

void SimpleSolver::output(const std::string &dir) {
    std::string tec = dir + "/tec";
    ::mkdir(tec.c_str(), 0755);  // the reference expects tec/ to exist
    char name[64];
    std::snprintf(name, sizeof name, "/res%04lu.dat", output_counter++);
    const long n = fd.nc;
    std::vector<std::vector<double>> h(10, std::vector<double>((size_t)n));
    const char *names[10] = {"P", "U", "V", "W", "R", "T", "VisLam", "VisTur", "TE", "ED"};
    for (int k = 0; k < 10; ++k) get_field(names[k], h[k].data(), n);
    TecFields f;
    f.P = h[0].data(); f.U = h[1].data(); f.V = h[2].data(); f.W = h[3].data(); f.R = h[4].data();
    f.T = h[5].data(); f.VisLam = h[6].data(); f.VisTur = h[7].data(); f.TE = h[8].data(); f.ED = h[9].data();
    std::vector<double> ts;
    if (cs.has_solid) {
        ts.resize((size_t)sd.nc);
        get_field("solid_T", ts.data(), sd.nc);
        f.solid_T = ts.data();
    }
    write_tecplot(cs, tec + name, f);
}

void SimpleSolver::volume_average(const std::string &dir, double t, int out_iter) {
    const long n = fd.nc;
    std::vector<double> R((size_t)n), P((size_t)n), T((size_t)n);
    get_field("R", R.data(), n);
    get_field("P", P.data(), n);
    get_field("T", T.data(), n);
    append_tot_line(cs, dir + "/tot.dat", t, out_iter, R.data(), P.data(), T.data());
}

double SimpleSolver::spmv_timing(const std::string &which, bool fp32, int reps, bool steady) {
    const DomainDev *d = &fd;
    const DevBuf<double> *v = nullptr;
    if (which == "mom") v = &f.Amom;
    else if (which == "p") v = &f.Ap;
    else if (which == "scalar") v = &f.As;
    else if (which == "solid" && cs.has_solid) { d = &sd; v = &s.As; }
    else throw CaseError{"spmv_timing: unknown matrix " + which};
    if (reps < 1) reps = 1;
    const SellDev &A = d->A;
    const size_t n = (size_t)A.n;
    DevBuf<double> x64(n), y64(n);
    DevBuf<float> x32(n), y32(n), v32;
    DevBuf<unsigned char> flush((size_t)256 << 20);
    DevBuf<unsigned> sink(1);
    DevBuf<int> err(1);
    err.zero(st);
    const bool ring = spmv_variant() == SPMV_RING;
    SYSU_CUDA(cudaMemsetAsync(flush.get(), 1, flush.size(), st));
    fill_sweep_x((long)n, x64.get(), x32.get(), st);
    if (fp32) {
        v32.alloc((size_t)A.nnz);
        sell_to_fp32(A, v->get(), v32.get(), st);
    }
    double total = 0.0;
    if (steady) {
        // products back to back, alternating between the matrix (values, column
        // indices, slice table) with x, y and a copy of all of them: 2 x 152 MB
        // (FP64, 2M rows) streamed in turn, more than the L2 holds, so every product
        // reads its operands from HBM as a product inside an iterative solve does,
        // without the launch ramp and tail a single timed product carries
        SellDev B;
        B.n = A.n;
        B.nslices = A.nslices;
        B.wmax = A.wmax;
        B.nnz = A.nnz;
        B.nnz_true = A.nnz_true;
        B.sl_ptr.alloc(A.sl_ptr.size());
        B.sl_w.alloc(A.sl_w.size());
        B.col.alloc(A.col.size());
        SYSU_CUDA(cudaMemcpyAsync(B.sl_ptr.get(), A.sl_ptr.get(), sizeof(int) * A.sl_ptr.size(), cudaMemcpyDeviceToDevice, st));
        SYSU_CUDA(cudaMemcpyAsync(B.sl_w.get(), A.sl_w.get(), sizeof(int) * A.sl_w.size(), cudaMemcpyDeviceToDevice, st));
        SYSU_CUDA(cudaMemcpyAsync(B.col.get(), A.col.get(), sizeof(int) * A.col.size(), cudaMemcpyDeviceToDevice, st));
        DevBuf<double> v64b, x64b(n), y64b(n);
        DevBuf<float> v32b, x32b(n), y32b(n);
        fill_sweep_x((long)n, x64b.get(), x32b.get(), st);
        if (fp32) {
            v32b.alloc((size_t)A.nnz);
            SYSU_CUDA(cudaMemcpyAsync(v32b.get(), v32.get(), sizeof(float) * A.nnz, cudaMemcpyDeviceToDevice, st));
        } else {
            v64b.alloc((size_t)A.nnz);
            SYSU_CUDA(cudaMemcpyAsync(v64b.get(), v->get(), sizeof(double) * A.nnz, cudaMemcpyDeviceToDevice, st));
        }
        auto product = [&](int k) {
            const bool second = k & 1;
            const SellDev &M = second ? B : A;
            if (ring && fp32) spmv_ring32(M, second ? v32b.get() : v32.get(), second ? x32b.get() : x32.get(),
                                          second ? y32b.get() : y32.get(), err.get(), st);
            else if (ring) spmv_ring(M, second ? v64b.get() : v->get(), second ? x64b.get() : x64.get(),
                                     second ? y64b.get() : y64.get(), err.get(), st);
            else if (fp32) spmv_stream32(M, second ? v32b.get() : v32.get(), second ? x32b.get() : x32.get(),
                                         second ? y32b.get() : y32.get(), st);
            else spmv_stream(M, second ? v64b.get() : v->get(), second ? x64b.get() : x64.get(),
                             second ? y64b.get() : y64.get(), st);
        };
        const int K = 2 * std::max(reps, 2);
        for (int k = 0; k < 4; ++k) product(k);  // warm-up
        SYSU_CUDA(cudaEventRecord(ev[4], st));
        for (int k = 0; k < K; ++k) product(k);
        SYSU_CUDA(cudaEventRecord(ev[5], st));
        SYSU_CUDA(cudaEventSynchronize(ev[5]));
        float ms = 0.f;
        SYSU_CUDA(cudaEventElapsedTime(&ms, ev[4], ev[5]));
        int e = 0;
        SYSU_CUDA(cudaMemcpy(&e, err.get(), sizeof(int), cudaMemcpyDeviceToHost));
        if (e != 0) throw CaseError{"spmv_timing: a bounded wait of the ring SpMV gave up"};
        return ms / K;
    }
    for (int k = 0; k < reps + 1; ++k) {
        l2_flush_read(flush.get(), flush.size(), sink.get(), st);
        SYSU_CUDA(cudaEventRecord(ev[4], st));
        if (ring && fp32) spmv_ring32(A, v32.get(), x32.get(), y32.get(), err.get(), st);
        else if (ring) spmv_ring(A, v->get(), x64.get(), y64.get(), err.get(), st);
        else if (fp32) spmv_stream32(A, v32.get(), x32.get(), y32.get(), st);
        else spmv_stream(A, v->get(), x64.get(), y64.get(), st);
        SYSU_CUDA(cudaEventRecord(ev[5], st));
        SYSU_CUDA(cudaEventSynchronize(ev[5]));
        float ms = 0.f;
        SYSU_CUDA(cudaEventElapsedTime(&ms, ev[4], ev[5]));
        if (k > 0) total += ms;  // the first product warms up
    }
    int e = 0;
    SYSU_CUDA(cudaMemcpy(&e, err.get(), sizeof(int), cudaMemcpyDeviceToHost));
    if (e != 0) throw CaseError{"spmv_timing: a bounded wait of the ring SpMV gave up"};
    return total / reps;
}

// ---------------------------------------------------------------------------
// Field access by the reference's member names.  kind: 0 cell, 1 cell gradient
// (3 per cell, interleaved like double** rows), 2 face (reference face order),
// 3 boundary record.
DevBuf<double> *SimpleSolver::field_ptr(const std::string &name, int &kind, bool &solid) {
    solid = false;
    std::string nm = name;
    if (nm.rfind("solid_", 0) == 0) {
        if (!cs.has_solid) return nullptr;
        solid = true;
        nm = nm.substr(6);
        FieldSet &fs = s;
        static const std::map<std::string, std::pair<int, int>> sm = {
            {"T", {0, 0}}, {"R", {0, 1}}, {"diffCoef", {0, 2}}, {"dPhidX", {1, 3}}, {"BTem", {3, 4}}, {"Bq", {3, 5}}};
        auto it = sm.find(nm);
        if (it == sm.end()) return nullptr;
        kind = it->second.first;
        DevBuf<double> *tab[] = {&fs.T, &fs.R, &fs.diff, &fs.dPhi, &fs.BTem, &fs.Bq};
        return tab[it->second.second];
    }
    struct E { const char *n; int kind; DevBuf<double> FieldSet::*p; };
    static const E tab[] = {
        {"U", 0, &FieldSet::U}, {"V", 0, &FieldSet::V}, {"W", 0, &FieldSet::W}, {"P", 0, &FieldSet::P},
        {"R", 0, &FieldSet::R}, {"T", 0, &FieldSet::T}, {"TE", 0, &FieldSet::TE}, {"ED", 0, &FieldSet::ED},
        {"VisLam", 0, &FieldSet::VisLam}, {"VisTur", 0, &FieldSet::VisTur}, {"Apr", 0, &FieldSet::Apr},
        {"dUdX", 1, &FieldSet::dU}, {"dVdX", 1, &FieldSet::dV}, {"dWdX", 1, &FieldSet::dW},
        {"dPdX", 1, &FieldSet::dP}, {"dPhidX", 1, &FieldSet::dPhi},
        {"RUFace", 2, &FieldSet::RUFace},
        {"BRo", 3, &FieldSet::BRo}, {"BU", 3, &FieldSet::BU}, {"BV", 3, &FieldSet::BV}, {"BW", 3, &FieldSet::BW},
        {"BPre", 3, &FieldSet::BPre}, {"BTem", 3, &FieldSet::BTem}, {"BTE", 3, &FieldSet::BTE},
        {"BED", 3, &FieldSet::BED}, {"Bq", 3, &FieldSet::Bq},
        {"dp", 0, &FieldSet::xp}, {"bp", 0, &FieldSet::bp},
        {"b3", 4, &FieldSet::b3}, {"x3", 4, &FieldSet::x3}, {"bs", 0, &FieldSet::bs},
    };
    for (const E &e : tab)
        if (nm == e.n) {
            kind = e.kind;
            return &(f.*(e.p));
        }
    return nullptr;
}

long SimpleSolver::field_size(const std::string &name) const {
    int kind;
    bool solid;
    DevBuf<double> *b = const_cast<SimpleSolver *>(this)->field_ptr(name, kind, solid);
    if (!b) return -1;
    const DomainDev &d = solid ? sd : fd;
    switch (kind) {
    case 0: return d.nc;
    case 1: return 3L * d.nc;
    case 2: return d.nf;
    case 4: return 3L * d.nc;
    default: return d.B;
    }
}

// Host <-> device field transfers: straight asynchronous copies for cell and
// record fields (DMA when the host buffer is pinned, e.g. from
// sysu_host_alloc), reordering on the device through a staging buffer for
// gradients and face fluxes.
void SimpleSolver::get_field(const std::string &name, double *out, long n) {
    int kind;
    bool solid;
    DevBuf<double> *b = field_ptr(name, kind, solid);
    if (!b) throw CaseError{"unknown field " + name};
    long sz = field_size(name);
    if (n != sz) throw CaseError{"field " + name + " has " + std::to_string(sz) + " values"};
    const DomainDev &d = solid ? sd : fd;
    const double *src = b->get();
    if (kind == 1 || kind == 2) {
        if (io_stage.size() < (size_t)sz) io_stage.alloc((size_t)sz);
        if (kind == 1) launch_soa3_to_aos3(io_stage.get(), b->get(), d.nc, st);
        else launch_scatter(io_stage.get(), b->get(), d.d_int2ref.get(), d.nf, st);
        src = io_stage.get();
    }
    if (sz) SYSU_CUDA(cudaMemcpyAsync(out, src, sizeof(double) * (size_t)sz, cudaMemcpyDeviceToHost, st));
    SYSU_CUDA(cudaStreamSynchronize(st));
}

void SimpleSolver::set_field(const std::string &name, const double *in, long n) {
    int kind;
    bool solid;
    DevBuf<double> *b = field_ptr(name, kind, solid);
    if (!b) throw CaseError{"unknown field " + name};
    long sz = field_size(name);
    if (n != sz) throw CaseError{"field " + name + " has " + std::to_string(sz) + " values"};
    const DomainDev &d = solid ? sd : fd;
    if (kind == 1 || kind == 2) {
        if (io_stage.size() < (size_t)sz) io_stage.alloc((size_t)sz);
        if (sz) SYSU_CUDA(cudaMemcpyAsync(io_stage.get(), in, sizeof(double) * (size_t)sz, cudaMemcpyHostToDevice, st));
        if (kind == 1) launch_aos3_to_soa3(b->get(), io_stage.get(), d.nc, st);
        else launch_gather(b->get(), io_stage.get(), d.d_int2ref.get(), d.nf, st);
    } else if (sz) {
        SYSU_CUDA(cudaMemcpyAsync(b->get(), in, sizeof(double) * (size_t)sz, cudaMemcpyHostToDevice, st));
    }
    SYSU_CUDA(cudaStreamSynchronize(st));
}

}  // namespace sysu
