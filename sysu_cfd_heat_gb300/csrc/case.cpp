// param.in parser, MSH reader, face builder, fluid/solid split and geometry.
// Compiled with -ffp-contract=off so that the geometry formulas round exactly
// like the reference's (which is built in ISO C++ mode, without contraction).
#include "case.hpp"
#include "parallel.hpp"

#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <unordered_map>

namespace sysu {

namespace {

[[noreturn]] void fail(const std::string &m) { throw CaseError{m}; }

std::string trim(const std::string &s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) ++b;
    while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
    return s.substr(b, e - b);
}

double to_f(const std::string &s) { return std::atof(s.c_str()); }
int to_i(const std::string &s) { return std::atoi(s.c_str()); }

}  // namespace

// readparamfile.cpp:10-260.  Same keywords, same quirks: a line is skipped only
// when it starts with "//" or has length 1 (a CRLF blank line), so an empty LF
// line is the unknown keyword "" and an error; unknown keywords are errors.
Params parse_params(const std::string &path) {
    std::ifstream fin(path);
    if (!fin) fail("param file can not found : " + path);
    Params p;
    std::string str;
    while (std::getline(fin, str)) {
        if (str.size() >= 2 && str[0] == '/' && str[1] == '/') continue;
        if (str.size() == 1) continue;
        std::vector<std::string> kw;
        {
            std::string cur;
            for (char c : str) {
                if (c != ',') cur.push_back(c);
                else {
                    kw.push_back(trim(cur));
                    cur.clear();
                }
            }
            kw.push_back(trim(cur));
        }
        int ikey = (int)kw.size() - 1;
        while (kw.size() < 20) kw.push_back("");
        const std::string &k = kw[0];
        if (k == "gridfile") {
            p.gridfile = kw[1];
        } else if (k == "steady") {
            p.steady = true;
            p.max_step = to_i(kw[1]);
            p.residual_steady = to_f(kw[2]);
        } else if (k == "transient") {
            p.steady = false;
            p.dt = to_f(kw[1]);
            p.total_time = to_f(kw[2]);
            if (kw[3] == "Euler") p.time_scheme = 1;
            else if (kw[3] == "Dual") p.time_scheme = 2;
            else fail("no such unsteady time scheme!");
            if (ikey >= 4) p.max_outer_step = to_i(kw[4]);
        } else if (k == "energy") {
            if (kw[1] == "on") p.solve_energy = true;
            else if (kw[1] == "off") p.solve_energy = false;
            else fail("energy key word is wrong");
        } else if (k == "density") {
            p.density_model = to_i(kw[1]);
        } else if (k == "turbulence") {
            if (kw[1] == "no") p.tur_model = 0;
            else if (kw[1] == "ke") p.tur_model = 1;
            else fail("turbulence key word is wrong");
        } else if (k == "gravity") {
            for (int g = 0; g < 3; ++g) p.gravity[g] = to_f(kw[1 + g]);
        } else if (k == "PressureRef") {
            p.pressure_reference = to_f(kw[1]);
            if (!kw[2].empty()) p.cell_pressure_ref = to_i(kw[2]) - 1;
        } else if (k == "relaxation") {
            p.urf[0] = p.urf[1] = p.urf[2] = to_f(kw[1]);
            p.urf[3] = to_f(kw[2]);
            p.urf[4] = to_f(kw[3]);
        } else if (k == "limiter") {
            if (kw[1] == "no") p.limiter = 0;
            else if (kw[1] == "Barth") p.limiter = 1;
            else if (kw[1] == "MLP") p.limiter = 2;
            else if (kw[1] == "WENO") p.limiter = 3;
            else fail("error in limiter definition");
        } else if (k == "initflow") {
            p.initflow.assign((size_t)std::max(ikey, 0), 0.0);
            for (int i = 1; i <= ikey; ++i) p.initflow[i - 1] = to_f(kw[i]);
            p.has_initflow = true;
        } else if (k == "bound") {
            int bid = to_i(kw[1]);
            if (p.regions.count(bid)) fail("repeating bid found : " + std::to_string(bid));
            if (bid == 0) fail("bid == 0 is illegal");
            Region r;
            if (kw[2] == "Twall") {
                r.name = "Twall"; r.type1 = 1; r.type2 = 0; r.fixedValue = to_f(kw[3]);
            } else if (kw[2] == "Hwall") {
                r.name = "Hwall"; r.type1 = 1; r.type2 = 1; r.fixedValue = to_f(kw[3]);
            } else if (kw[2] == "sym") {
                r.name = "sym"; r.type1 = 4; r.type2 = 0; r.fixedValue = 0.0;
            } else if (kw[2] == "inlet") {
                r.name = "inlet"; r.type1 = 2; r.type2 = 0;
                for (int i = 0; i < 6; ++i) r.initvalues[i] = to_f(kw[3 + i]);
                if (p.tur_model == 1) {  // only when "turbulence, ke" came earlier
                    r.initvalues[6] = to_f(kw[9]);
                    r.initvalues[7] = to_f(kw[10]);
                }
            } else if (kw[2] == "outlet") {
                r.name = "outlet"; r.type1 = 3; r.type2 = 0; r.fixedValue = to_f(kw[3]);
            } else {
                fail("unknown boundry type in bound : " + kw[2]);
            }
            p.regions[bid] = r;
        } else if (k == "volumn") {
            int bid = to_i(kw[1]);
            if (p.regions.count(bid)) fail("repeating bid found");
            if (bid == 0) fail("bid == 0 is ilegal");
            Region r;
            if (kw[2] == "fluid") { r.type1 = 5; r.type2 = 0; }
            else if (kw[2] == "solid") { r.type1 = 5; r.type2 = 1; }
            else fail("unknown boundry type in bound : " + kw[2]);
            r.name = kw[3];
            for (int i = 4; i <= ikey && i - 4 < 10; ++i) r.initvalues[i - 4] = to_f(kw[i]);
            p.regions[bid] = r;
        } else if (k == "output") {
            p.noutput = to_i(kw[1]);
            p.outputformat = (kw[2] == "vtk") ? 1 : 0;
        } else if (k == "3dheatconduction") {
            p.heat_conduction = true;
        } else {
            fail("no such command:  : " + k);
        }
    }
    if (p.steady) p.max_outer_step = p.max_step;  // navier.cpp:21-24
    return p;
}

// ---------------------------------------------------------------------------
// Gmsh MSH 2.x ASCII, Preprocessor.cpp:13-146: six tokens are skipped before the
// node count, two after the nodes; then n_elem elements with 2 or 3 tags.
namespace {
struct Tok {
    const char *p, *e;
    bool skip_ws() {
        while (p < e && std::isspace((unsigned char)*p)) ++p;
        return p < e;
    }
    void word() {
        if (!skip_ws()) fail("unexpected end of mesh file");
        while (p < e && !std::isspace((unsigned char)*p)) ++p;
    }
    long integer() {
        if (!skip_ws()) fail("unexpected end of mesh file");
        char *end;
        long v = std::strtol(p, &end, 10);
        if (end == p) fail("bad integer in mesh file");
        p = end;
        return v;
    }
    double real() {
        if (!skip_ws()) fail("unexpected end of mesh file");
        char *end;
        double v = std::strtod(p, &end);
        if (end == p) fail("bad number in mesh file");
        p = end;
        return v;
    }
};
}  // namespace

namespace {

constexpr int ELEM_NODES[8] = {0, 2, 3, 4, 4, 8, 6, 5};

// One element record (the reference's Preprocessor.cpp:96-146 reading and the
// 8-vertex cell form of its element types); "" or the error message.
template <class Sink>
std::string read_element(Tok &t, long nv, Sink &m) {
    int v[8], tag[10];
    t.integer();
    long et = t.integer();
    long ntags = t.integer();
    if (ntags != 2 && ntags != 3) return "element with other than 2 or 3 tags";
    if (et < 1 || et > 7) return "Unknown element type !!!";
    for (long q = 0; q < ntags; ++q) tag[q] = (int)t.integer();
    for (int q = 0; q < ELEM_NODES[et]; ++q) {
        long vi = t.integer() - 1;
        if (vi < 0 || vi >= nv) return "element references a missing vertex";
        v[q] = (int)vi;
    }
    if (et == 2 || et == 3) {
        m.bnd_rid.push_back(tag[0]);
        int f4[4] = {v[0], v[1], v[2], et == 2 ? v[2] : v[3]};
        m.bnd_vert.insert(m.bnd_vert.end(), f4, f4 + 4);
    } else if (et >= 4 && et <= 7) {
        int c[8];
        if (et == 4) {  // tet
            c[0] = v[0]; c[1] = v[1]; c[2] = v[2]; c[3] = v[2];
            c[4] = c[5] = c[6] = c[7] = v[3];
        } else if (et == 5) {
            for (int q = 0; q < 8; ++q) c[q] = v[q];
        } else if (et == 6) {  // prism
            c[0] = v[0]; c[1] = v[1]; c[2] = v[2]; c[3] = v[2];
            c[4] = v[3]; c[5] = v[4]; c[6] = v[5]; c[7] = v[5];
        } else {  // pyramid
            for (int q = 0; q < 4; ++q) c[q] = v[q];
            c[4] = c[5] = c[6] = c[7] = v[4];
        }
        m.cell_rid.push_back(tag[0]);
        m.cell_vert.insert(m.cell_vert.end(), c, c + 8);
    } else {
        return "Unknown element type !!!";
    }
    return "";
}

RawMesh read_msh_seq(const std::string &buf) {
    Tok t{buf.data(), buf.data() + buf.size()};
    for (int i = 0; i < 6; ++i) t.word();
    RawMesh m;
    long nv = t.integer();
    if (nv <= 0) fail("mesh has no vertices");
    m.nv = (int)nv;
    m.vert.resize((size_t)nv * 3);
    for (long i = 0; i < nv; ++i) {
        t.integer();
        for (int k = 0; k < 3; ++k) m.vert[(size_t)i * 3 + k] = t.real();
    }
    t.word();
    t.word();
    long ne = t.integer();
    if (ne <= 0) fail("mesh has no elements");
    m.cell_vert.reserve((size_t)ne * 8);
    for (long i = 0; i < ne; ++i) {
        std::string e = read_element(t, nv, m);
        if (!e.empty()) fail(e);
    }
    return m;
}

// Split [b, e) into T pieces that start at line beginnings.
std::vector<const char *> line_splits(const char *b, const char *e, int T) {
    std::vector<const char *> cut{b};
    for (int k = 1; k < T; ++k) {
        const char *p = b + (e - b) * k / T;
        if (p < cut.back()) p = cut.back();
        while (p < e && *p != '\n') ++p;
        if (p < e) ++p;
        cut.push_back(p);
    }
    cut.push_back(e);
    return cut;
}

const char *find_marker(const char *b, const char *e, const char *marker) {
    size_t len = std::strlen(marker);
    const char *p = std::search(b, e, marker, marker + len);
    return p == e ? nullptr : p;
}

// The same reading with the node and element sections split over threads at
// line boundaries (Gmsh writes one record per line).  Returns false when the
// file does not have that layout or any record fails; the caller then reads it
// sequentially, which reports the reference's error.
bool read_msh_par(const std::string &buf, int T, RawMesh &m) {
    const char *B = buf.data(), *E = B + buf.size();
    Tok t{B, E};
    for (int i = 0; i < 6; ++i) t.word();
    long nv = t.integer();
    if (nv <= 0) return false;
    const char *ns = t.p, *nend = find_marker(ns, E, "$EndNodes");
    if (!nend) return false;
    std::vector<const char *> cut = line_splits(ns, nend, T);
    std::vector<std::vector<double>> vparts(T);
    std::vector<int> vok(T, 1);
    parallel_chunks(T, T, [&](long k0, long k1, int) {
        for (long k = k0; k < k1; ++k) {
            Tok c{cut[k], cut[k + 1]};
            std::vector<double> &out = vparts[k];
            try {
                while (c.skip_ws()) {
                    c.integer();
                    for (int q = 0; q < 3; ++q) out.push_back(c.real());
                }
            } catch (...) {
                vok[k] = 0;
            }
        }
    });
    size_t nvals = 0;
    for (int k = 0; k < T; ++k) {
        if (!vok[k]) return false;
        nvals += vparts[k].size();
    }
    if (nvals != (size_t)nv * 3) return false;
    m.nv = (int)nv;
    m.vert.clear();
    m.vert.reserve(nvals);
    for (auto &v : vparts) m.vert.insert(m.vert.end(), v.begin(), v.end());
    Tok t2{nend, E};
    t2.word();
    t2.word();
    long ne = t2.integer();
    if (ne <= 0) return false;
    const char *es = t2.p, *eend = find_marker(es, E, "$EndElements");
    if (!eend) return false;
    cut = line_splits(es, eend, T);
    std::vector<RawMesh> parts(T);
    std::vector<long> cnt(T, 0);
    parallel_chunks(T, T, [&](long k0, long k1, int) {
        for (long k = k0; k < k1; ++k) {
            Tok c{cut[k], cut[k + 1]};
            try {
                while (c.skip_ws()) {
                    if (!read_element(c, nv, parts[k]).empty()) {
                        vok[k] = 0;
                        break;
                    }
                    ++cnt[k];
                }
            } catch (...) {
                vok[k] = 0;
            }
        }
    });
    long total = 0;
    size_t ncv = 0, nbv = 0;
    for (int k = 0; k < T; ++k) {
        if (!vok[k]) return false;
        total += cnt[k];
        ncv += parts[k].cell_vert.size();
        nbv += parts[k].bnd_vert.size();
    }
    if (total != ne) return false;
    m.cell_vert.reserve(ncv);
    m.cell_rid.reserve(ncv / 8);
    m.bnd_vert.reserve(nbv);
    m.bnd_rid.reserve(nbv / 4);
    for (RawMesh &p : parts) {
        m.cell_vert.insert(m.cell_vert.end(), p.cell_vert.begin(), p.cell_vert.end());
        m.cell_rid.insert(m.cell_rid.end(), p.cell_rid.begin(), p.cell_rid.end());
        m.bnd_vert.insert(m.bnd_vert.end(), p.bnd_vert.begin(), p.bnd_vert.end());
        m.bnd_rid.insert(m.bnd_rid.end(), p.bnd_rid.begin(), p.bnd_rid.end());
    }
    return true;
}

}  // namespace

double *setup_phases() {
    static thread_local double ph[5] = {0, 0, 0, 0, 0};
    return ph;
}

namespace {
double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

RawMesh read_msh(const std::string &path) {
    double t0 = now_s();
    struct Stamp {
        double t0;
        ~Stamp() { setup_phases()[0] = now_s() - t0; }
    } stamp{t0};
    setup_phases()[4] = host_threads();
    std::ifstream f(path, std::ios::binary);
    if (!f) fail("grid file not found : " + path);
    std::string buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    int T = host_threads();
    if (T > 1 && buf.size() > (size_t)(1 << 20)) {
        RawMesh m;
        bool ok = false;
        try {
            ok = read_msh_par(buf, T, m);
        } catch (...) {
            ok = false;
        }
        if (ok) return m;
    }
    return read_msh_seq(buf);
}

// ---------------------------------------------------------------------------
// Face construction in the reference's order (Preprocessor.cpp:181-299):
// boundary elements become faces 0..nb-1; then every cell visits its six
// local faces in a fixed order, skipping degenerate ones, and either creates a
// face (with the vertices in the visiting order) or claims an existing one.
// The node->face table of the reference is replaced by a hash of the sorted
// vertex set.
namespace {

struct FaceKey {
    int v[4];
    bool operator==(const FaceKey &o) const {
        return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2] && v[3] == o.v[3];
    }
};
struct FaceKeyHash {
    size_t operator()(const FaceKey &k) const {
        uint64_t h = 1469598103934665603ull;
        for (int i = 0; i < 4; ++i) {
            h ^= (uint64_t)(uint32_t)k.v[i];
            h *= 1099511628211ull;
        }
        return (size_t)(h ^ (h >> 29));
    }
};

FaceKey key_of(int a, int b, int c, int d) {
    int s[4] = {a, b, c, d};
    std::sort(s, s + 4);
    FaceKey k;
    int n = 0;
    for (int i = 0; i < 4; ++i)
        if (i == 0 || s[i] != s[i - 1]) k.v[n++] = s[i];
    for (; n < 4; ++n) k.v[n] = -1;
    return k;
}

struct Topo {
    int nv = 0;
    std::vector<double> vert;
    std::vector<int> cell_vert, cell_rid, cell_nface, cell_face;
    std::vector<int> face_vert, face_c1, face_c2, face_bnd;
    std::vector<int> bnd_face, bnd_rid;
};

void create_faces_seq(const RawMesh &m, Topo &t) {
    int nc = m.ncell(), nb = m.nbnd();
    t.nv = m.nv;
    t.vert = m.vert;
    t.cell_vert = m.cell_vert;
    t.cell_rid = m.cell_rid;
    t.cell_nface.assign(nc, 0);
    t.cell_face.assign((size_t)nc * 6, -1);
    t.bnd_rid = m.bnd_rid;
    t.bnd_face.resize(nb);
    size_t est = (size_t)nb + (size_t)nc * 3;
    t.face_vert.reserve(est * 4);
    t.face_c1.reserve(est);
    t.face_c2.reserve(est);
    t.face_bnd.reserve(est);
    std::unordered_map<FaceKey, int, FaceKeyHash> table;
    table.reserve(est * 2);
    for (int i = 0; i < nb; ++i) {
        int f = (int)t.face_c1.size();
        t.bnd_face[i] = f;
        const int *bv = &m.bnd_vert[(size_t)i * 4];
        t.face_vert.insert(t.face_vert.end(), bv, bv + 4);
        t.face_bnd.push_back(i);
        t.face_c1.push_back(-10);
        t.face_c2.push_back(-10);
        table.emplace(key_of(bv[0], bv[1], bv[2], bv[3]), f);
    }
    static const int lf[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                 {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}};
    for (int ic = 0; ic < nc; ++ic) {
        const int *cv = &m.cell_vert[(size_t)ic * 8];
        for (int q = 0; q < 6; ++q) {
            int n1 = cv[lf[q][0]], n2 = cv[lf[q][1]], n3 = cv[lf[q][2]], n4 = cv[lf[q][3]];
            int irepeat = 0;
            if (n1 == n2 || n1 == n3 || n1 == n4) ++irepeat;
            if (n2 == n3 || n2 == n4) ++irepeat;
            if (n3 == n4) ++irepeat;
            if (irepeat > 1) continue;
            FaceKey k = key_of(n1, n2, n3, n4);
            auto it = table.find(k);
            int fid;
            if (it == table.end()) {
                fid = (int)t.face_c1.size();
                int fv[4] = {n1, n2, n3, n4};
                t.face_vert.insert(t.face_vert.end(), fv, fv + 4);
                t.face_c1.push_back(ic);
                t.face_c2.push_back(-20);  // set by the second cell
                t.face_bnd.push_back(-10);
                table.emplace(k, fid);
            } else {
                fid = it->second;
                if (t.face_bnd[fid] >= 0) {
                    if (t.face_c1[fid] == -10) t.face_c1[fid] = ic;
                    else if (t.face_c2[fid] == -10) t.face_c2[fid] = ic;
                    else fail("boundary face shared by more than two cells");
                } else {
                    if (t.face_c2[fid] != -20) fail("interior face shared by more than two cells");
                    t.face_c2[fid] = ic;
                }
            }
            if (t.cell_nface[ic] >= 6) fail("cell with more than six faces");
            t.cell_face[(size_t)ic * 6 + t.cell_nface[ic]++] = fid;
        }
    }
    // NavierStokesSolver::CheckAndAllocate (navier.cpp:497-503): every face is
    // either interior or a marked boundary face.
    for (size_t f = 0; f < t.face_c2.size(); ++f) {
        if (t.face_c2[f] == -20) fail("error in face right hand side (a boundary face is not marked)");
        if (t.face_bnd[f] >= 0 && t.face_c1[f] < 0) fail("boundary element that bounds no cell");
    }
}

// The same face construction over threads.  Every candidate face gets a slot in
// visiting order (boundary elements 0..nb-1, then nb + 6 ic + q); the candidates
// are distributed over hash shards by key, each shard thread scans all slots in
// order and claims the ones of its keys, so every key sees its visits in the
// reference's order.  A face's id is the rank of its first visit among all first
// visits (a prefix sum), which is the order in which the sequential loop creates
// faces.  Returns false on anything the sequential loop would report (the caller
// reruns it for the exact message).
bool create_faces_par(const RawMesh &m, Topo &t, int T) {
    const int nc = m.ncell(), nb = m.nbnd();
    const long S = (long)nb + 6L * nc;
    static const int lf[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                 {1, 2, 6, 5}, {3, 2, 6, 7}, {0, 3, 7, 4}};
    auto slot_verts = [&](long s, int *v) {
        if (s < nb) {
            const int *bv = &m.bnd_vert[(size_t)s * 4];
            for (int k = 0; k < 4; ++k) v[k] = bv[k];
            return true;
        }
        long r = s - nb;
        int ic = (int)(r / 6), q = (int)(r % 6);
        const int *cv = &m.cell_vert[(size_t)ic * 8];
        int n1 = cv[lf[q][0]], n2 = cv[lf[q][1]], n3 = cv[lf[q][2]], n4 = cv[lf[q][3]];
        int irepeat = 0;
        if (n1 == n2 || n1 == n3 || n1 == n4) ++irepeat;
        if (n2 == n3 || n2 == n4) ++irepeat;
        if (n3 == n4) ++irepeat;
        v[0] = n1; v[1] = n2; v[2] = n3; v[3] = n4;
        return irepeat <= 1;
    };
    std::vector<FaceKey> key((size_t)S);
    std::vector<uint32_t> hsh((size_t)S);
    const uint32_t INVALID = 0xFFFFFFFFu;
    FaceKeyHash H;
    parallel_chunks(S, T, [&](long b, long e, int) {
        int v[4];
        for (long s = b; s < e; ++s) {
            if (!slot_verts(s, v)) {
                hsh[s] = INVALID;
                continue;
            }
            key[s] = key_of(v[0], v[1], v[2], v[3]);
            hsh[s] = (uint32_t)(H(key[s]) & 0x7FFFFFFFu);
        }
    });
    // shard tables: open addressing, per entry the first slot, c1, c2, bnd
    struct Entry {
        FaceKey k;
        int first, c1, c2, bnd;
    };
    std::vector<int> first_of((size_t)S, -1);
    std::vector<std::vector<Entry>> tab(T);
    std::vector<int> bad(T, 0);
    parallel_chunks(T, T, [&](long t0, long t1, int) {
        for (long sh = t0; sh < t1; ++sh) {
            long mine = 0;
            for (long s = 0; s < S; ++s)
                if (hsh[s] != INVALID && (long)(hsh[s] % (uint32_t)T) == sh) ++mine;
            size_t cap = 16;
            while (cap < (size_t)mine * 2) cap <<= 1;
            std::vector<Entry> &E = tab[sh];
            E.assign(cap, Entry{{{-3, -3, -3, -3}}, -1, 0, 0, 0});
            const size_t mask = cap - 1;
            for (long s = 0; s < S && !bad[sh]; ++s) {
                uint32_t h = hsh[s];
                if (h == INVALID || (long)(h % (uint32_t)T) != sh) continue;
                size_t i = (h / (uint32_t)T) & mask;
                while (E[i].first >= 0 && !(E[i].k == key[s])) i = (i + 1) & mask;
                Entry &en = E[i];
                if (s < nb) {
                    if (en.first >= 0) {  // duplicate boundary element
                        bad[sh] = 1;
                        break;
                    }
                    en.k = key[s];
                    en.first = (int)s;
                    en.c1 = -10;
                    en.c2 = -10;
                    en.bnd = (int)s;
                    first_of[s] = (int)s;
                    continue;
                }
                int ic = (int)((s - nb) / 6);
                if (en.first < 0) {
                    en.k = key[s];
                    en.first = (int)s;
                    en.c1 = ic;
                    en.c2 = -20;
                    en.bnd = -10;
                } else if (en.bnd >= 0) {
                    if (en.c1 == -10) en.c1 = ic;
                    else if (en.c2 == -10) en.c2 = ic;
                    else { bad[sh] = 1; break; }
                } else {
                    if (en.c2 != -20) { bad[sh] = 1; break; }
                    en.c2 = ic;
                }
                first_of[s] = en.first;
            }
        }
    });
    for (int sh = 0; sh < T; ++sh)
        if (bad[sh]) return false;
    // face ids: exclusive prefix count of first visits, in slot order
    std::vector<int> fid((size_t)S, -1);
    std::vector<long> part(T + 1, 0);
    parallel_chunks(S, T, [&](long b, long e, int k) {
        long c = 0;
        for (long s = b; s < e; ++s)
            if (first_of[s] == s) ++c;
        part[k + 1] = c;
    });
    for (int k = 0; k < T; ++k) part[k + 1] += part[k];
    const long nf = part[T];
    parallel_chunks(S, T, [&](long b, long e, int k) {
        long c = part[k];
        for (long s = b; s < e; ++s)
            if (first_of[s] == s) fid[s] = (int)c++;
    });
    t.nv = m.nv;
    t.vert = m.vert;
    t.cell_vert = m.cell_vert;
    t.cell_rid = m.cell_rid;
    t.bnd_rid = m.bnd_rid;
    t.bnd_face.resize(nb);
    for (int i = 0; i < nb; ++i) t.bnd_face[i] = i;
    t.face_vert.assign((size_t)nf * 4, 0);
    t.face_c1.assign(nf, 0);
    t.face_c2.assign(nf, 0);
    t.face_bnd.assign(nf, 0);
    parallel_chunks(T, T, [&](long t0, long t1, int) {
        for (long sh = t0; sh < t1; ++sh)
            for (const Entry &en : tab[sh]) {
                if (en.first < 0) continue;
                int f = fid[en.first];
                int v[4];
                slot_verts(en.first, v);
                for (int k = 0; k < 4; ++k) t.face_vert[(size_t)f * 4 + k] = v[k];
                t.face_c1[f] = en.c1;
                t.face_c2[f] = en.c2;
                t.face_bnd[f] = en.bnd;
            }
    });
    t.cell_nface.assign(nc, 0);
    t.cell_face.assign((size_t)nc * 6, -1);
    parallel_chunks(nc, T, [&](long b, long e, int) {
        for (long ic = b; ic < e; ++ic) {
            int k = 0;
            for (int q = 0; q < 6; ++q) {
                long s = nb + ic * 6 + q;
                if (hsh[s] == INVALID) continue;
                t.cell_face[(size_t)ic * 6 + k++] = fid[first_of[s]];
            }
            t.cell_nface[ic] = k;
        }
    });
    for (long f = 0; f < nf; ++f) {
        if (t.face_c2[f] == -20) return false;
        if (t.face_bnd[f] >= 0 && t.face_c1[f] < 0) return false;
    }
    return true;
}

void create_faces(const RawMesh &m, Topo &t) {
    int T = host_threads();
    if (T > 1 && m.ncell() >= 20000) {
        Topo p;
        if (create_faces_par(m, p, T)) {
            t = std::move(p);
            return;
        }
    }
    create_faces_seq(m, t);
}

// findCoupledBoundary (Preprocessor.cpp:308-438) for the cells in new2old.
void extract_domain(const Topo &t, const std::vector<int> &new2old, int coupled_rid, Domain &d) {
    int nc = (int)new2old.size();
    std::unordered_map<int, int> o2nv, o2nf;
    o2nv.reserve((size_t)nc * 2);
    o2nf.reserve((size_t)nc * 4);
    d.nc = nc;
    d.cell_vert.assign((size_t)nc * 8, 0);
    d.cell_rid.resize(nc);
    d.cell_nface.resize(nc);
    d.cell_face.assign((size_t)nc * 6, -1);
    d.vert.clear();
    int nv = 0;
    for (int i = 0; i < nc; ++i) {
        int o = new2old[i];
        d.cell_rid[i] = t.cell_rid[o];
        d.cell_nface[i] = t.cell_nface[o];
        for (int j = 0; j < 8; ++j) {
            int iv = t.cell_vert[(size_t)o * 8 + j];
            auto it = o2nv.find(iv);
            if (it != o2nv.end()) {
                d.cell_vert[(size_t)i * 8 + j] = it->second;
            } else {
                for (int k = 0; k < 3; ++k) d.vert.push_back(t.vert[(size_t)iv * 3 + k]);
                d.cell_vert[(size_t)i * 8 + j] = nv;
                o2nv.emplace(iv, nv++);
            }
        }
    }
    d.nv = nv;
    d.face_vert.clear();
    d.face_c1.clear();
    d.face_c2.clear();
    d.face_bnd.clear();
    int nf = 0;
    for (int i = 0; i < nc; ++i) {
        int o = new2old[i];
        for (int j = 0; j < t.cell_nface[o]; ++j) {
            int of = t.cell_face[(size_t)o * 6 + j];
            auto it = o2nf.find(of);
            if (it != o2nf.end()) {
                d.face_c2[it->second] = i;
                d.cell_face[(size_t)i * 6 + j] = it->second;
            } else {
                for (int k = 0; k < 4; ++k) d.face_vert.push_back(o2nv.at(t.face_vert[(size_t)of * 4 + k]));
                d.face_c1.push_back(i);
                d.face_c2.push_back(-10);
                d.face_bnd.push_back(t.face_bnd[of]);
                d.cell_face[(size_t)i * 6 + j] = nf;
                o2nf.emplace(of, nf++);
            }
        }
    }
    d.nf = nf;
    d.bnd_face.clear();
    d.bnd_rid.clear();
    int nb = 0;
    for (int f = 0; f < nf; ++f) {
        if (d.face_c2[f] < 0 && d.face_bnd[f] >= 0) {
            d.bnd_rid.push_back(t.bnd_rid[d.face_bnd[f]]);
            d.bnd_face.push_back(f);
            d.face_bnd[f] = nb++;
        }
    }
    d.ncb = nb;
    for (int f = 0; f < nf; ++f) {
        if (d.face_c2[f] < 0 && d.face_bnd[f] < 0) {
            d.bnd_rid.push_back(coupled_rid);
            d.bnd_face.push_back(f);
            d.face_bnd[f] = nb++;
        }
    }
    d.nb = nb;
}

}  // namespace

// ---------------------------------------------------------------------------
// CycasSolver::CellFaceInfo, BasicSolver.cpp:317-512, with the same expression
// order (vec_dot/vec_len accumulate left to right from 0).
namespace {
inline void vminus(double *o, const double *a, const double *b) {
    for (int i = 0; i < 3; ++i) o[i] = a[i] - b[i];
}
inline double vdot(const double *a, const double *b) {
    double s = 0.;
    for (int i = 0; i < 3; ++i) s += a[i] * b[i];
    return s;
}
inline double vlen(const double *a) {
    double s = 0.;
    for (int i = 0; i < 3; ++i) s += a[i] * a[i];
    return std::sqrt(s);
}
inline void vcross(double *a, const double *b, const double *c) {
    a[0] = b[1] * c[2] - b[2] * c[1];
    a[1] = -b[0] * c[2] + b[2] * c[0];
    a[2] = b[0] * c[1] - b[1] * c[0];
}
double tri_area(const double *x1, const double *x2, const double *x3) {
    double v1[3], v2[3];
    vminus(v1, x2, x1);
    vminus(v2, x3, x1);
    double a1 = v1[1] * v2[2] - v1[2] * v2[1];
    double a2 = -v1[0] * v2[2] + v1[2] * v2[0];
    double a3 = v1[0] * v2[1] - v1[1] * v2[0];
    return 0.5 * std::sqrt(a1 * a1 + a2 * a2 + a3 * a3);
}
double tet_vol(const double *x1, const double *x2, const double *x3, const double *x4) {
    double v1[3], d1[3], d2[3], d3[3];
    vminus(d1, x2, x1);
    vminus(d2, x3, x1);
    vminus(d3, x4, x1);
    vcross(v1, d1, d2);
    return 1. / 6. * std::fabs(vdot(v1, d3));
}
}  // namespace

// Each loop runs over threads (static chunks); a check that fails reports the
// lowest failing index of its loop, the one the sequential loop meets first.
void cell_face_info(Domain &d) {
    const int T = d.nc >= 20000 ? host_threads() : 1;
    const double *V = d.vert.data();
    auto X = [&](int iv) { return V + (size_t)iv * 3; };
    const long NONE = -1;
    std::vector<long> firstbad(T);
    auto reset_bad = [&]() { std::fill(firstbad.begin(), firstbad.end(), NONE); };
    auto note_bad = [&](int k, long i) {
        if (firstbad[k] == NONE || i < firstbad[k]) firstbad[k] = i;
    };
    auto lowest_bad = [&]() {
        long lo = NONE;
        for (long b : firstbad)
            if (b != NONE && (lo == NONE || b < lo)) lo = b;
        return lo;
    };
    d.cell_x.assign((size_t)d.nc * 3, 0.0);
    d.cell_vol.assign(d.nc, 0.0);
    parallel_chunks(d.nc, T, [&](long b, long e, int) {
        for (long i = b; i < e; ++i) {
            const int *cv = &d.cell_vert[(size_t)i * 8];
            for (int j = 0; j < 3; ++j)
                d.cell_x[(size_t)i * 3 + j] =
                    1. / 8. * (X(cv[0])[j] + X(cv[1])[j] + X(cv[2])[j] + X(cv[3])[j] + X(cv[4])[j] +
                               X(cv[5])[j] + X(cv[6])[j] + X(cv[7])[j]);
        }
    });
    d.face_x.assign((size_t)d.nf * 3, 0.0);
    d.face_n.assign((size_t)d.nf * 3, 0.0);
    d.face_area.assign(d.nf, 0.0);
    d.face_lambda.assign(d.nf, 0.0);
    d.face_rlencos.assign(d.nf, 0.0);
    d.face_xpac.assign((size_t)d.nf * 3, 0.0);
    d.face_xnac.assign((size_t)d.nf * 3, 0.0);
    reset_bad();
    parallel_chunks(d.nf, T, [&](long b, long e, int k) {
        for (long i = b; i < e; ++i) {
            const int *fv = &d.face_vert[(size_t)i * 4];
            const double *p1 = X(fv[0]), *p2 = X(fv[1]), *p3 = X(fv[2]), *p4 = X(fv[3]);
            double area1 = tri_area(p1, p2, p4);
            double area2 = tri_area(p2, p3, p4);
            double xc1[3], xc2[3];
            for (int j = 0; j < 3; ++j) {
                xc1[j] = 1. / 3 * (p1[j] + p2[j] + p4[j]);
                xc2[j] = 1. / 3 * (p2[j] + p3[j] + p4[j]);
            }
            double *fx = &d.face_x[(size_t)i * 3];
            for (int j = 0; j < 3; ++j) fx[j] = (area1 * xc1[j] + area2 * xc2[j]) / (area1 + area2);
            double dx1[3], dx2[3], dx[3];
            vminus(dx1, p1, p3);
            vminus(dx2, p2, p4);
            double *fn = &d.face_n[(size_t)i * 3];
            vcross(fn, dx1, dx2);
            for (int j = 0; j < 3; ++j) fn[j] = 0.5 * fn[j];
            int ic = d.face_c1[i];
            vminus(dx, fx, &d.cell_x[(size_t)ic * 3]);
            if (vdot(fn, dx) < 0.)
                for (int j = 0; j < 3; ++j) fn[j] = -fn[j];
            d.face_area[i] = vlen(fn);
            if (std::fabs((area1 + area2 - d.face_area[i]) / d.face_area[i]) > 1.e-4) note_bad(k, i);
            int ic1 = d.face_c1[i], ic2 = d.face_c2[i];
            if (ic2 >= 0) {
                vminus(dx1, fx, &d.cell_x[(size_t)ic1 * 3]);
                vminus(dx2, fx, &d.cell_x[(size_t)ic2 * 3]);
                double r1 = vlen(dx1), r2 = vlen(dx2);
                d.face_lambda[i] = r2 / (r1 + r2);
            } else {
                d.face_lambda[i] = 1.;
            }
        }
    });
    if (lowest_bad() != NONE) fail("face " + std::to_string(lowest_bad()) + " area is not correct (non-planar face)");
    d.cell_nbr.assign((size_t)d.nc * 6, -100);
    reset_bad();
    parallel_chunks(d.nc, T, [&](long b, long e, int k) {
        for (long i = b; i < e; ++i) {
            const int *cv = &d.cell_vert[(size_t)i * 8];
            double xv[8][3];
            for (int q = 0; q < 8; ++q)
                for (int j = 0; j < 3; ++j) xv[q][j] = X(cv[q])[j];
            double V1 = tet_vol(xv[0], xv[1], xv[3], xv[5]);
            double V2 = tet_vol(xv[0], xv[4], xv[3], xv[5]);
            double V3 = tet_vol(xv[3], xv[4], xv[7], xv[5]);
            double V4 = tet_vol(xv[1], xv[2], xv[3], xv[6]);
            double V5 = tet_vol(xv[1], xv[5], xv[3], xv[6]);
            double V6 = tet_vol(xv[7], xv[3], xv[5], xv[6]);
            d.cell_vol[i] = V1 + V2 + V3 + V4 + V5 + V6;
            double c[6][3];
            for (int j = 0; j < 3; ++j) {
                c[0][j] = 0.25 * (xv[0][j] + xv[1][j] + xv[3][j] + xv[5][j]);
                c[1][j] = 0.25 * (xv[0][j] + xv[4][j] + xv[3][j] + xv[5][j]);
                c[2][j] = 0.25 * (xv[3][j] + xv[4][j] + xv[7][j] + xv[5][j]);
                c[3][j] = 0.25 * (xv[1][j] + xv[2][j] + xv[3][j] + xv[6][j]);
                c[4][j] = 0.25 * (xv[1][j] + xv[5][j] + xv[3][j] + xv[6][j]);
                c[5][j] = 0.25 * (xv[7][j] + xv[3][j] + xv[5][j] + xv[6][j]);
            }
            double Vsum = V1 + V2 + V3 + V4 + V5 + V6;
            for (int j = 0; j < 3; ++j)
                d.cell_x[(size_t)i * 3 + j] = 1. / Vsum *
                    (V1 * c[0][j] + V2 * c[1][j] + V3 * c[2][j] + V4 * c[3][j] + V5 * c[4][j] + V6 * c[5][j]);
            if (!(d.cell_vol[i] > 0.)) note_bad(k, i);
            for (int j = 0; j < d.cell_nface[i]; ++j) {
                int f = d.cell_face[(size_t)i * 6 + j];
                int nc = d.face_c1[f];
                if (nc == i) nc = d.face_c2[f];
                d.cell_nbr[(size_t)i * 6 + j] = nc;
            }
        }
    });
    if (lowest_bad() != NONE) fail("error in cell volume calculation: cell " + std::to_string(lowest_bad()));
    d.bnd_distance.assign(d.nb, 0.0);
    reset_bad();
    parallel_chunks(d.nb, T, [&](long b, long e, int k) {
        for (long i = b; i < e; ++i) {
            int jf = d.bnd_face[i], jc = d.face_c1[jf];
            double dx[3];
            vminus(dx, &d.face_x[(size_t)jf * 3], &d.cell_x[(size_t)jc * 3]);
            d.bnd_distance[i] = vdot(dx, &d.face_n[(size_t)jf * 3]) / d.face_area[jf];
            if (d.bnd_distance[i] < 0.) note_bad(k, i);
        }
    });
    if (lowest_bad() != NONE) fail("wall distance is negative." + std::to_string(lowest_bad()));
    parallel_chunks(d.nf, T, [&](long b, long e, int) {
        for (long i = b; i < e; ++i) {
            int ic1 = d.face_c1[i], ic2 = d.face_c2[i];
            const double *fx = &d.face_x[(size_t)i * 3];
            const double *fn = &d.face_n[(size_t)i * 3];
            double area = d.face_area[i];
            double dx[3];
            if (ic2 < 0) vminus(dx, fx, &d.cell_x[(size_t)ic1 * 3]);
            else vminus(dx, &d.cell_x[(size_t)ic2 * 3], &d.cell_x[(size_t)ic1 * 3]);
            d.face_rlencos[i] = area / (vdot(dx, fn) / area);
            if (ic2 >= 0) {
                double ss;
                vminus(dx, fx, &d.cell_x[(size_t)ic1 * 3]);
                ss = vdot(dx, fn) / area;
                for (int j = 0; j < 3; ++j) dx[j] = ss * fn[j] / area;
                vminus(&d.face_xpac[(size_t)i * 3], fx, dx);
                vminus(dx, fx, &d.cell_x[(size_t)ic2 * 3]);
                ss = vdot(dx, fn) / area;
                for (int j = 0; j < 3; ++j) dx[j] = ss * fn[j] / area;
                vminus(&d.face_xnac[(size_t)i * 3], fx, dx);
            }
        }
    });
}

void build_case(const RawMesh &raw, Case &cs) {
    Topo t;
    double t0 = now_s();
    create_faces(raw, t);
    double t1 = now_s();
    setup_phases()[1] = t1 - t0;
    const Params &p = cs.params;
    auto to_domain = [&](const std::vector<int> &new2old, int crid, Domain &d) { extract_domain(t, new2old, crid, d); };
    if (!p.heat_conduction) {
        // buildSolver without heat conduction hands the global mesh over as is
        Domain &d = cs.fluid;
        d.nv = t.nv;
        d.vert = std::move(t.vert);
        d.nc = raw.ncell();
        d.cell_vert = std::move(t.cell_vert);
        d.cell_rid = std::move(t.cell_rid);
        d.cell_nface = std::move(t.cell_nface);
        d.cell_face = std::move(t.cell_face);
        d.nf = (int)t.face_c1.size();
        d.face_vert = std::move(t.face_vert);
        d.face_c1 = std::move(t.face_c1);
        d.face_c2 = std::move(t.face_c2);
        d.face_bnd = std::move(t.face_bnd);
        d.nb = raw.nbnd();
        d.ncb = d.nb;
        d.bnd_face = std::move(t.bnd_face);
        d.bnd_rid = std::move(t.bnd_rid);
        cs.has_solid = false;
    } else {
        // Preprocessor.cpp:453-512: a coupled wall region takes the first unused id
        int crid = -1;
        for (int i = 0; i <= (int)p.regions.size(); ++i)
            if (!p.regions.count(i)) { crid = i; break; }
        Region cr;
        cr.name = "coupled boundary";
        cr.type1 = 1;
        cr.type2 = 2;
        cs.params.regions[crid] = cr;
        cs.coupled_rid = crid;
        std::vector<int> nf, ns;
        for (int i = 0; i < raw.ncell(); ++i) {
            auto it = p.regions.find(raw.cell_rid[i]);
            if (it == p.regions.end()) fail("no such rid for body, rid: : " + std::to_string(raw.cell_rid[i]));
            if (it->second.type1 != 5) fail("body should has rid 5");
            (it->second.type2 == 0 ? nf : ns).push_back(i);
        }
        to_domain(nf, crid, cs.fluid);
        to_domain(ns, crid, cs.solid);
        cs.has_solid = true;
    }
    // region checks the reference makes while running (navier_bc.cpp:52-53,
    // navier.cpp:141): fail early instead
    auto check_domain = [&](const Domain &d, bool solid) {
        for (int i = 0; i < d.nb; ++i) {
            auto it = cs.params.regions.find(d.bnd_rid[i]);
            if (it == cs.params.regions.end())
                fail("boundary id " + std::to_string(d.bnd_rid[i]) + " has no bound keyword");
            int ty = it->second.type1;
            if (solid ? !(ty == 1 || ty == 4) : !(ty >= 1 && ty <= 4))
                fail("no such boundary type in velocity bc: " + std::to_string(ty));
        }
        for (int i = 0; i < d.nc; ++i) {
            auto it = cs.params.regions.find(d.cell_rid[i]);
            if (it == cs.params.regions.end() || it->second.type1 != 5 || it->second.type2 != (solid ? 1 : 0))
                fail(std::string(solid ? "solid" : "fluid") + " cell with a region that is not a " +
                     (solid ? "solid" : "fluid") + " volumn");
        }
    };
    double t2 = now_s();
    setup_phases()[2] = t2 - t1;
    cell_face_info(cs.fluid);
    check_domain(cs.fluid, false);
    if (cs.has_solid) {
        cell_face_info(cs.solid);
        check_domain(cs.solid, true);
        if (cs.fluid.nb - cs.fluid.ncb != cs.solid.nb - cs.solid.ncb)
            fail("fluid and solid have different numbers of coupled faces");
    }
    setup_phases()[3] = now_s() - t2;
}

}  // namespace sysu
