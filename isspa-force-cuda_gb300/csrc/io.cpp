// io.cpp -- readers for the reference's input formats and the host-side
// system object.  Semantics follow the reference readers line by line
// (fixed-width Amber fields, unit conversions, index shifts) so that the same
// files produce the same arrays; errors are reported as status codes instead
// of exit() or silent garbage.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "host_system.h"
#include "philox.h"

namespace {

struct LineFile {
    FILE *f = nullptr;
    explicit LineFile(const char *path) : f(std::fopen(path, "r")) {}
    ~LineFile() {
        if (f) std::fclose(f);
    }
    bool ok() const { return f != nullptr; }
    bool next(std::string &line) {
        line.clear();
        char buf[4096];
        if (!std::fgets(buf, sizeof buf, f)) return false;
        line = buf;
        // long lines: keep reading until newline
        while (!line.empty() && line.back() != '\n') {
            if (!std::fgets(buf, sizeof buf, f)) break;
            line += buf;
        }
        return true;
    }
};

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

// Fixed-width field k of width w, parsed like atoi/atof of the reference's
// strncpy'd token.  Returns false when the line is too short.
bool field_int(const std::string &line, int k, int w, int &out) {
    size_t at = (size_t)k * w;
    if (at >= line.size()) return false;
    std::string t = line.substr(at, w);
    if (trim(t).empty()) return false;
    out = std::atoi(t.c_str());
    return true;
}
bool field_dbl(const std::string &line, int k, int w, double &out) {
    size_t at = (size_t)k * w;
    if (at >= line.size()) return false;
    std::string t = line.substr(at, w);
    if (trim(t).empty()) return false;
    out = std::atof(t.c_str());
    return true;
}

// Name of a "%FLAG NAME" line, or "" (read_prmtop.cpp:62-64).
std::string flag_name(const std::string &line) {
    if (line.compare(0, 5, "%FLAG") != 0) return "";
    size_t a = 5;
    while (a < line.size() && std::isspace((unsigned char)line[a])) ++a;
    size_t b = a;
    while (b < line.size() && !std::isspace((unsigned char)line[b])) ++b;
    return line.substr(a, b - a);
}

// Read `count` fixed-width values, `per_line` per line (the reference's
// nLines loops), after skipping the %FORMAT line.
template <typename T, typename Conv>
int read_block(LineFile &lf, int count, int per_line, int width, std::vector<T> &out, Conv conv) {
    std::string line;
    if (!lf.next(line)) return ISSPA_ERR_PARSE;  // format line
    out.resize(count);
    int n = 0;
    while (n < count) {
        if (!lf.next(line)) return ISSPA_ERR_PARSE;
        for (int k = 0; k < per_line && n < count; ++k) {
            double v;
            if (!field_dbl(line, k, width, v)) return ISSPA_ERR_PARSE;
            out[n++] = conv(v);
        }
    }
    return ISSPA_OK;
}
int read_ints(LineFile &lf, int count, std::vector<int> &out) {
    std::string line;
    if (!lf.next(line)) return ISSPA_ERR_PARSE;
    out.resize(count);
    int n = 0;
    while (n < count) {
        if (!lf.next(line)) return ISSPA_ERR_PARSE;
        for (int k = 0; k < 10 && n < count; ++k) {
            int v;
            if (!field_int(line, k, 8, v)) return ISSPA_ERR_PARSE;
            out[n++] = v;
        }
    }
    return ISSPA_OK;
}
int read_floats(LineFile &lf, int count, std::vector<double> &out) {
    return read_block(lf, count, 5, 16, out, [](double v) { return v; });
}

// strtok-like split used by the reference's `key = value # comment` parsers
// (config_class.cpp:26-28): leading delimiters are skipped, so text after a
// leading '#' is parsed as well.
bool split_key_value(const std::string &raw, std::string &key, std::string &val) {
    auto tok = [](const std::string &s, size_t &pos, char delim) -> std::string {
        while (pos < s.size() && s[pos] == delim) ++pos;
        if (pos >= s.size()) return std::string("\x01");
        size_t e = s.find(delim, pos);
        std::string t = s.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
        pos = e == std::string::npos ? s.size() : e + 1;
        return t;
    };
    size_t p = 0;
    std::string first = tok(raw, p, '#');
    if (first == "\x01") return false;
    size_t q = 0;
    std::string k = tok(first, q, '=');
    if (k == "\x01") return false;
    key = trim(k);
    std::string v = tok(first, q, '=');
    val = v == "\x01" ? std::string() : trim(v.substr(0, 80));
    return true;
}

bool starts(const std::string &key, const char *name) {
    return std::strncmp(key.c_str(), name, std::strlen(name)) == 0;
}

void copy_name(char *dst, const std::string &v) {
    std::snprintf(dst, 512, "%s", v.c_str());
}

std::string join_path(const char *base, const char *p) {
    if (!base || !*base || p[0] == '/') return p;
    std::string b(base);
    if (b.back() != '/') b += '/';
    return b + p;
}

}  // namespace

extern "C" {

int isspa_read_run_config(const char *path, isspa_run_config *c) {
    if (!path || !c) return ISSPA_ERR_ARG;
    LineFile lf(path);
    if (!lf.ok()) return ISSPA_ERR_IO;
    std::memset(c, 0, sizeof *c);
    std::string line, key, val;
    while (lf.next(line)) {
        if (!split_key_value(line, key, val)) continue;
        // same test order as config_class.cpp:30-117 (prefix matches)
        if (starts(key, "prmtop")) copy_name(c->prmtop, val);
        else if (starts(key, "isspaPrmtop")) copy_name(c->isspa_prmtop, val);
        else if (starts(key, "posFile")) copy_name(c->pos_out, val);
        else if (starts(key, "posRstFile")) copy_name(c->pos_rst_file, val);
        else if (starts(key, "velFile")) copy_name(c->vel_out, val);
        else if (starts(key, "velRstFile")) copy_name(c->vel_rst_file, val);
        else if (starts(key, "forFile")) copy_name(c->for_out, val);
        else if (starts(key, "inputCoord")) copy_name(c->input_coord, val);
        else if (starts(key, "nMC")) c->n_mc = std::atoi(val.c_str());
        else if (starts(key, "temperature")) c->temperature = (float)std::atof(val.c_str());
        else if (starts(key, "seed")) c->seed = (int)std::atof(val.c_str());
        else if (starts(key, "cutoff")) c->cutoff = (float)std::atof(val.c_str());
        else if (starts(key, "dielectric")) c->eps = (float)std::atof(val.c_str());
        else if (starts(key, "nSteps")) c->n_steps = std::atoi(val.c_str());
        else if (starts(key, "deltaWrite")) c->delta_write = std::atoi(val.c_str());
        else if (starts(key, "boxLength")) c->box = (float)std::atof(val.c_str());
        else if (starts(key, "pnu")) {
            c->pnu = (float)std::atof(val.c_str());
            c->pnu_set = 1;
        } else if (starts(key, "velRst")) c->vel_rst = std::atoi(val.c_str());
        else if (starts(key, "inputVel")) copy_name(c->input_vel, val);
        else if (starts(key, "US")) c->us = std::atoi(val.c_str());
        else if (starts(key, "usCfgFile")) copy_name(c->us_cfg, val);
    }
    // config_class.cpp:123-126
    c->dt_ps = 0.002f;
    c->dt = c->dt_ps * 20.455f;
    c->kT = c->temperature * 0.00198717f;
    return ISSPA_OK;
}

int isspa_read_prmtop(const char *path, float eps, isspa_host_system **out) {
    if (!path || !out) return ISSPA_ERR_ARG;
    LineFile lf(path);
    if (!lf.ok()) return ISSPA_ERR_IO;
    auto *s = new isspa_host_system();
    int nBondH = 0, nBondnH = 0, nAngH = 0, nAngnH = 0, nDihH = 0, nDihnH = 0, exclLen = 0;
    bool got_ptr = false, got_charge = false, got_mass = false, got_type = false, got_excl = false,
         got_nbp = false, got_lja = false, got_ljb = false;
    const float sqrtEps = std::sqrt(eps);  // read_prmtop.cpp:57
    std::string line;
    std::vector<int> tmp;
    std::vector<double> dv;
    int rc = ISSPA_OK;
    while (rc == ISSPA_OK && lf.next(line)) {
        std::string flag = flag_name(line);
        if (flag.empty()) continue;
        if (flag == "POINTERS") {  // :66-112
            std::string l1, l2;
            if (!lf.next(line) || !lf.next(l1) || !lf.next(l2)) { rc = ISSPA_ERR_PARSE; break; }
            int v[8], w[8];
            for (int k = 0; k < 8; ++k)
                if (!field_int(l1, k, 8, v[k])) { rc = ISSPA_ERR_PARSE; break; }
            for (int k = 0; k < 8 && rc == ISSPA_OK; ++k)
                if (!field_int(l2, k, 8, w[k])) { rc = ISSPA_ERR_PARSE; break; }
            if (rc) break;
            s->n_atoms = v[0];
            s->n_lj_types = v[1];
            nBondH = v[2]; nBondnH = v[3]; nAngH = v[4]; nAngnH = v[5]; nDihH = v[6]; nDihnH = v[7];
            exclLen = w[0];
            s->n_bond_types = w[5]; s->n_angle_types = w[6]; s->n_dih_types = w[7];
            if (s->n_atoms <= 0 || s->n_lj_types <= 0 || exclLen < 0 || nBondH < 0 || nBondnH < 0 ||
                nAngH < 0 || nAngnH < 0 || nDihH < 0 || nDihnH < 0) { rc = ISSPA_ERR_PARSE; break; }
            s->pos.assign(4 * (size_t)s->n_atoms, 0.f);
            s->vel.assign(4 * (size_t)s->n_atoms, 0.f);
            s->raw_mass.assign(s->n_atoms, 0.f);
            s->bond_params.assign(2 * (size_t)std::max(s->n_bond_types, 0), 0.f);
            s->angle_params.assign(2 * (size_t)std::max(s->n_angle_types, 0), 0.f);
            s->dih_params.assign(4 * (size_t)std::max(s->n_dih_types, 0), 0.f);
            s->scaled14.assign(2 * (size_t)std::max(s->n_dih_types, 0), 0.f);
            s->lj_ab.assign(2 * (size_t)(s->n_lj_types * (s->n_lj_types + 1) / 2), 0.f);
            lf.next(line);  // line 4 (read_prmtop.cpp:106)
            got_ptr = true;
            continue;
        }
        if (!got_ptr) continue;
        const int N = s->n_atoms;
        if (flag == "CHARGE") {  // :113-129
            if ((rc = read_floats(lf, N, dv))) break;
            for (int i = 0; i < N; ++i) s->pos[4 * i + 3] = (float)dv[i] / sqrtEps;
            got_charge = true;
        } else if (flag == "MASS") {  // :130-150
            if ((rc = read_floats(lf, N, dv))) break;
            for (int i = 0; i < N; ++i) {
                float m = (float)dv[i];
                s->raw_mass[i] = m;
                s->vel[4 * i + 3] = m < 2.0f ? 12.0f : m;
            }
            got_mass = true;
        } else if (flag == "ATOM_TYPE_INDEX") {  // :151-166
            if ((rc = read_ints(lf, N, tmp))) break;
            s->lj_type.resize(N);
            for (int i = 0; i < N; ++i) s->lj_type[i] = tmp[i] - 1;
            got_type = true;
        } else if (flag == "NUMBER_EXCLUDED_ATOMS") {  // :167-186 (cumulative)
            if ((rc = read_ints(lf, N, tmp))) break;
            s->n_excl_cum.resize(N);
            int acc = 0;
            for (int i = 0; i < N; ++i) s->n_excl_cum[i] = (acc += tmp[i]);
        } else if (flag == "NONBONDED_PARM_INDEX") {  // :187-203
            if ((rc = read_ints(lf, s->n_lj_types * s->n_lj_types, tmp))) break;
            s->nb_parm_index.resize(tmp.size());
            for (size_t i = 0; i < tmp.size(); ++i) s->nb_parm_index[i] = tmp[i] - 1;
            got_nbp = true;
        } else if (flag == "BOND_EQUIL_VALUE" || flag == "BOND_FORCE_CONSTANT") {  // :204-237
            if ((rc = read_floats(lf, s->n_bond_types, dv))) break;
            bool k = flag == "BOND_FORCE_CONSTANT";
            for (int i = 0; i < s->n_bond_types; ++i)
                s->bond_params[2 * i + (k ? 0 : 1)] = k ? (float)dv[i] * 2.0f : (float)dv[i];
        } else if (flag == "ANGLE_EQUIL_VALUE" || flag == "ANGLE_FORCE_CONSTANT") {  // :238-271
            if ((rc = read_floats(lf, s->n_angle_types, dv))) break;
            bool k = flag == "ANGLE_FORCE_CONSTANT";
            for (int i = 0; i < s->n_angle_types; ++i)
                s->angle_params[2 * i + (k ? 0 : 1)] = k ? (float)dv[i] * 2.0f : (float)dv[i];
        } else if (flag == "DIHEDRAL_PERIODICITY" || flag == "DIHEDRAL_FORCE_CONSTANT" ||
                   flag == "DIHEDRAL_PHASE") {  // :273-320
            if ((rc = read_floats(lf, s->n_dih_types, dv))) break;
            int c = flag == "DIHEDRAL_PERIODICITY" ? 0 : (flag == "DIHEDRAL_FORCE_CONSTANT" ? 1 : 2);
            for (int i = 0; i < s->n_dih_types; ++i) s->dih_params[4 * i + c] = (float)dv[i];
        } else if (flag == "SCEE_SCALE_FACTOR" || flag == "SCNB_SCALE_FACTOR") {  // :321-352
            if ((rc = read_floats(lf, s->n_dih_types, dv))) break;
            int c = flag == "SCEE_SCALE_FACTOR" ? 0 : 1;
            for (int i = 0; i < s->n_dih_types; ++i) s->scaled14[2 * i + c] = (float)dv[i];
        } else if (flag == "LENNARD_JONES_ACOEF" || flag == "LENNARD_JONES_BCOEF") {  // :353-384
            int n2 = s->n_lj_types * (s->n_lj_types + 1) / 2;
            if ((rc = read_floats(lf, n2, dv))) break;
            int c = flag == "LENNARD_JONES_ACOEF" ? 0 : 1;
            for (int i = 0; i < n2; ++i) s->lj_ab[2 * i + c] = (float)dv[i];
            (c ? got_ljb : got_lja) = true;
        } else if (flag == "BONDS_INC_HYDROGEN" || flag == "BONDS_WITHOUT_HYDROGEN") {  // :386-437
            bool h = flag == "BONDS_INC_HYDROGEN";
            int n = h ? nBondH : nBondnH, off = h ? 0 : nBondH;
            if ((rc = read_ints(lf, 3 * n, tmp))) break;
            s->bond_atoms.resize(3 * (size_t)(nBondH + nBondnH));
            for (int i = 0; i < n; ++i) {
                s->bond_atoms[3 * (off + i) + 0] = tmp[3 * i] / 3;
                s->bond_atoms[3 * (off + i) + 1] = tmp[3 * i + 1] / 3;
                s->bond_atoms[3 * (off + i) + 2] = tmp[3 * i + 2] - 1;
            }
        } else if (flag == "ANGLES_INC_HYDROGEN" || flag == "ANGLES_WITHOUT_HYDROGEN") {  // :439-492
            bool h = flag == "ANGLES_INC_HYDROGEN";
            int n = h ? nAngH : nAngnH, off = h ? 0 : nAngH;
            if ((rc = read_ints(lf, 4 * n, tmp))) break;
            s->angle_atoms.resize(4 * (size_t)(nAngH + nAngnH));
            for (int i = 0; i < n; ++i) {
                for (int k = 0; k < 3; ++k) s->angle_atoms[4 * (off + i) + k] = tmp[4 * i + k] / 3;
                s->angle_atoms[4 * (off + i) + 3] = tmp[4 * i + 3] - 1;
            }
        } else if (flag == "DIHEDRALS_INC_HYDROGEN" || flag == "DIHEDRALS_WITHOUT_HYDROGEN") {  // :494-545
            bool h = flag == "DIHEDRALS_INC_HYDROGEN";
            int n = h ? nDihH : nDihnH, off = h ? 0 : nDihH;
            if ((rc = read_ints(lf, 5 * n, tmp))) break;
            s->dih_atoms.resize(4 * (size_t)(nDihH + nDihnH));
            s->dih_types.resize(nDihH + nDihnH);
            for (int i = 0; i < n; ++i) {
                for (int k = 0; k < 4; ++k) s->dih_atoms[4 * (off + i) + k] = tmp[5 * i + k] / 3;
                s->dih_types[off + i] = tmp[5 * i + 4] - 1;
            }
        } else if (flag == "EXCLUDED_ATOMS_LIST") {  // :546-562
            if ((rc = read_ints(lf, exclLen, tmp))) break;
            s->excl_list.resize(exclLen);
            for (int i = 0; i < exclLen; ++i) s->excl_list[i] = tmp[i] - 1;
            got_excl = true;
        }
    }
    if (rc == ISSPA_OK) {
        if (!got_ptr || !got_charge || !got_mass || !got_type || !got_nbp || !got_lja || !got_ljb)
            rc = ISSPA_ERR_PARSE;
        if (s->n_excl_cum.empty()) s->n_excl_cum.assign(s->n_atoms, 0);
        if (!got_excl) s->excl_list.clear();
        if ((int)s->bond_atoms.size() != 3 * (nBondH + nBondnH)) s->bond_atoms.resize(3 * (size_t)(nBondH + nBondnH), 0);
        if ((int)s->angle_atoms.size() != 4 * (nAngH + nAngnH)) s->angle_atoms.resize(4 * (size_t)(nAngH + nAngnH), 0);
        if ((int)s->dih_types.size() != nDihH + nDihnH) {
            s->dih_atoms.resize(4 * (size_t)(nDihH + nDihnH), 0);
            s->dih_types.resize(nDihH + nDihnH, 0);
        }
    }
    if (rc == ISSPA_OK) {
        // range checks the reference never made
        const int N = s->n_atoms, nt = s->n_lj_types, ntt = nt * (nt + 1) / 2;
        for (int t : s->lj_type) if (t < 0 || t >= nt) rc = ISSPA_ERR_PARSE;
        for (int t : s->nb_parm_index) if (t < 0 || t >= ntt) rc = ISSPA_ERR_UNSUPPORTED;
        int prev = 0;
        for (int c : s->n_excl_cum) { if (c < prev || c > (int)s->excl_list.size()) rc = ISSPA_ERR_PARSE; prev = c; }
        for (size_t b = 0; b < s->bond_atoms.size() / 3; ++b) {
            const int *a = &s->bond_atoms[3 * b];
            if (a[0] < 0 || a[0] >= N || a[1] < 0 || a[1] >= N || a[2] < 0 || a[2] >= s->n_bond_types) rc = ISSPA_ERR_PARSE;
        }
        for (size_t b = 0; b < s->angle_atoms.size() / 4; ++b) {
            const int *a = &s->angle_atoms[4 * b];
            for (int k = 0; k < 3; ++k) if (a[k] < 0 || a[k] >= N) rc = ISSPA_ERR_PARSE;
            if (a[3] < 0 || a[3] >= s->n_angle_types) rc = ISSPA_ERR_PARSE;
        }
        for (size_t b = 0; b < s->dih_types.size(); ++b) {
            const int *a = &s->dih_atoms[4 * b];
            for (int k = 0; k < 4; ++k) if (std::abs(a[k]) >= N) rc = ISSPA_ERR_PARSE;
            if (s->dih_types[b] < 0 || s->dih_types[b] >= s->n_dih_types) rc = ISSPA_ERR_PARSE;
        }
    }
    if (rc != ISSPA_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return ISSPA_OK;
}

int isspa_read_isspatop(isspa_host_system *s, const char *path) {
    if (!s || !path) return ISSPA_ERR_ARG;
    LineFile lf(path);
    if (!lf.ok()) return ISSPA_ERR_IO;
    std::string line;
    int nAtoms = -1, nTypes = 0, nG = 0, nE = 0, nF = 0;
    bool got_types = false, got_rmax = false, got_g = false, got_e = false, got_f = false;
    std::vector<int> tmp;
    std::vector<double> dv;
    auto table = [&](int rows, std::vector<float> &tab, float &r0, float &dr) -> int {
        if (!lf.next(line)) return ISSPA_ERR_PARSE;  // format line
        tab.assign((size_t)nTypes * rows, 0.f);
        std::vector<double> r(rows);
        for (int i = 0; i < rows; ++i) {
            if (!lf.next(line)) return ISSPA_ERR_PARSE;
            double v;
            if (!field_dbl(line, 0, 16, v)) return ISSPA_ERR_PARSE;
            r[i] = v;
            for (int t = 0; t < nTypes; ++t) {
                if (!field_dbl(line, t + 1, 16, v)) return ISSPA_ERR_PARSE;
                tab[(size_t)t * rows + i] = (float)v;
            }
        }
        if (rows < 2) return ISSPA_ERR_PARSE;
        // isspa_class.cpp:137-138 etc.: min and bin size from the first two rows
        r0 = (float)r[0];
        dr = (float)r[1] - (float)r[0];
        if (!(dr > 0.f)) return ISSPA_ERR_PARSE;
        for (float v : tab) if (!std::isfinite(v)) return ISSPA_ERR_PARSE;
        return ISSPA_OK;
    };
    int rc = ISSPA_OK;
    while (rc == ISSPA_OK && lf.next(line)) {
        std::string flag = flag_name(line);
        if (flag.empty()) continue;
        // prefix matches as isspa_class.cpp:72-155
        if (flag.compare(0, 8, "POINTERS") == 0) {
            std::string l1;
            if (!lf.next(line) || !lf.next(l1)) { rc = ISSPA_ERR_PARSE; break; }
            if (!field_int(l1, 0, 8, nAtoms) || !field_int(l1, 1, 8, nTypes) || !field_int(l1, 2, 8, nG) ||
                !field_int(l1, 3, 8, nE) || !field_int(l1, 4, 8, nF)) { rc = ISSPA_ERR_PARSE; break; }
            if (nAtoms <= 0 || nTypes <= 0 || nG < 2 || nE < 2 || nF < 2) { rc = ISSPA_ERR_PARSE; break; }
        } else if (nAtoms < 0) {
            continue;
        } else if (flag.compare(0, 16, "ISSPA_TYPE_INDEX") == 0) {
            if ((rc = read_ints(lf, nAtoms, tmp))) break;
            s->isspa_type.resize(nAtoms);
            for (int i = 0; i < nAtoms; ++i) {
                s->isspa_type[i] = tmp[i] - 1;
                if (tmp[i] < 1 || tmp[i] > nTypes) rc = ISSPA_ERR_PARSE;
            }
            got_types = true;
        } else if (flag.compare(0, 10, "ISSPA_RMAX") == 0) {
            if ((rc = read_floats(lf, nTypes, dv))) break;
            s->rmax.resize(nTypes);
            for (int t = 0; t < nTypes; ++t) {
                s->rmax[t] = (float)dv[t];
                if (!(s->rmax[t] > 0.f)) rc = ISSPA_ERR_PARSE;
            }
            got_rmax = true;
        } else if (flag.compare(0, 15, "ISSPA_DENSITIES") == 0) {
            rc = table(nG, s->g_table, s->g_r0, s->g_dr);
            got_g = true;
        } else if (flag.compare(0, 12, "ISSPA_EFIELD") == 0) {
            rc = table(nE, s->e_table, s->e_r0, s->e_dr);
            got_e = true;
        } else if (flag.compare(0, 12, "ISSPA_FORCES") == 0) {
            rc = table(nF, s->f_table, s->f_r0, s->f_dr);
            got_f = true;
        }
    }
    if (rc == ISSPA_OK && !(got_types && got_rmax && got_g && got_e && got_f)) rc = ISSPA_ERR_PARSE;
    if (rc == ISSPA_OK && s->n_atoms && nAtoms != s->n_atoms) rc = ISSPA_ERR_PARSE;
    if (rc != ISSPA_OK) return rc;
    s->n_isspa_types = nTypes;
    s->n_g = nG;
    s->n_e = nE;
    s->n_f = nF;
    s->have_isspa = true;
    return ISSPA_OK;
}

int isspa_read_rst7(isspa_host_system *s, const char *path, int velocities) {
    if (!s || !path || s->n_atoms <= 0) return ISSPA_ERR_ARG;
    LineFile lf(path);
    if (!lf.ok()) return ISSPA_ERR_IO;
    std::string line;
    // atom_class.cpp:86-103: two header lines, then 6 values of 12 chars per line
    if (!lf.next(line) || !lf.next(line)) return ISSPA_ERR_PARSE;
    const int N = s->n_atoms;
    std::vector<float> tmp(3 * (size_t)N);
    int nLines = N / 2;
    for (int i = 0; i < nLines; ++i) {
        if (!lf.next(line)) return ISSPA_ERR_PARSE;
        for (int j = 0; j < 6; ++j) {
            double v;
            if (!field_dbl(line, j, 12, v)) return ISSPA_ERR_PARSE;
            tmp[6 * i + j] = (float)v;
        }
    }
    if (N % 2) {
        if (!lf.next(line)) return ISSPA_ERR_PARSE;
        for (int j = 0; j < 3; ++j) {
            double v;
            if (!field_dbl(line, j, 12, v)) return ISSPA_ERR_PARSE;
            tmp[6 * nLines + j] = (float)v;
        }
    }
    std::vector<float> &dst = velocities ? s->vel : s->pos;
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < 3; ++k) {
            if (!std::isfinite(tmp[3 * i + k])) return ISSPA_ERR_PARSE;
            dst[4 * i + k] = tmp[3 * i + k];
        }
    return ISSPA_OK;
}

int isspa_read_us_config(isspa_host_system *s, const char *path, char *cv_file_out, size_t cv_len) {
    if (!s || !path) return ISSPA_ERR_ARG;
    LineFile lf(path);
    if (!lf.ok()) return ISSPA_ERR_IO;
    std::string line, key, val, g1, g2, cv;
    bool have1 = false, have2 = false;
    while (lf.next(line)) {
        if (!split_key_value(line, key, val)) continue;
        // us_class.cpp:36-71
        if (starts(key, "k")) s->us_k = (float)std::atof(val.c_str());
        else if (starts(key, "x0")) s->us_x0 = (float)std::atof(val.c_str());
        else if (starts(key, "cvFile")) cv = val;
        else if (starts(key, "atomSelect1")) { g1 = val; have1 = true; }
        else if (starts(key, "atomSelect2")) { g2 = val; have2 = true; }
    }
    if (!have1 || !have2) return ISSPA_ERR_PARSE;
    s->bias_list.clear();
    auto parse = [&](const std::string &lst, int g) -> int {
        size_t p = 0;
        while (p <= lst.size()) {
            size_t e = lst.find(',', p);
            std::string t = trim(lst.substr(p, e == std::string::npos ? std::string::npos : e - p));
            if (!t.empty()) {
                int a = std::atoi(t.c_str()) - 1;  // us_class.cpp:86
                if (a < 0 || a >= s->n_atoms) return ISSPA_ERR_PARSE;
                s->bias_list.push_back(a);
                s->bias_list.push_back(g);
            }
            if (e == std::string::npos) break;
            p = e + 1;
        }
        return ISSPA_OK;
    };
    int rc = parse(g1, 0);
    if (rc == ISSPA_OK) rc = parse(g2, 1);
    if (rc != ISSPA_OK) return rc;
    s->us_on = 1;
    if (cv_file_out && cv_len) std::snprintf(cv_file_out, cv_len, "%s", cv.c_str());
    return ISSPA_OK;
}

int isspa_system_set_run(isspa_host_system *s, int n_mc, float box, float kT, float dt, float pnu,
                         uint64_t seed) {
    if (!s) return ISSPA_ERR_ARG;
    s->n_mc = n_mc;
    s->box = box;
    s->kT = kT;
    s->dt = dt;
    s->pnu = pnu;
    s->seed = seed;
    return ISSPA_OK;
}

int isspa_system_load(const isspa_run_config *c, const char *base, isspa_host_system **out) {
    if (!c || !out) return ISSPA_ERR_ARG;
    isspa_host_system *s = nullptr;
    float eps = c->eps > 0.f ? c->eps : 1.0f;
    int rc = isspa_read_prmtop(join_path(base, c->prmtop).c_str(), eps, &s);
    if (rc) return rc;
    isspa_system_set_run(s, c->n_mc, c->box, c->kT, c->dt, c->pnu_set ? c->pnu : 0.0f,
                         (uint64_t)(int64_t)c->seed);
    rc = isspa_read_isspatop(s, join_path(base, c->isspa_prmtop).c_str());
    if (!rc) rc = isspa_read_rst7(s, join_path(base, c->input_coord).c_str(), 0);
    if (!rc) {
        if (c->vel_rst == 1) rc = isspa_read_rst7(s, join_path(base, c->input_vel).c_str(), 1);
        else isspa::init_velocities(*s, (uint64_t)(int64_t)c->seed);
    }
    if (!rc && c->us == 1) rc = isspa_read_us_config(s, join_path(base, c->us_cfg).c_str(), nullptr, 0);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return ISSPA_OK;
}

int isspa_system_describe(const isspa_host_system *s, isspa_system_desc *d) {
    if (!s || !d) return ISSPA_ERR_ARG;
    std::memset(d, 0, sizeof *d);
    d->n_atoms = s->n_atoms;
    d->pos = s->pos.data();
    d->vel = s->vel.data();
    d->raw_mass = s->raw_mass.data();
    d->n_lj_types = s->n_lj_types;
    d->lj_type = s->lj_type.data();
    d->nb_parm_index = s->nb_parm_index.data();
    d->lj_ab = s->lj_ab.data();
    d->excl_len = (int)s->excl_list.size();
    d->n_excl_cum = s->n_excl_cum.data();
    d->excl_list = s->excl_list.data();
    d->n_bonds = (int)s->bond_atoms.size() / 3;
    d->bond_atoms = s->bond_atoms.data();
    d->n_bond_types = s->n_bond_types;
    d->bond_params = s->bond_params.data();
    d->n_angles = (int)s->angle_atoms.size() / 4;
    d->angle_atoms = s->angle_atoms.data();
    d->n_angle_types = s->n_angle_types;
    d->angle_params = s->angle_params.data();
    d->n_dihs = (int)s->dih_types.size();
    d->dih_atoms = s->dih_atoms.data();
    d->dih_types = s->dih_types.data();
    d->n_dih_types = s->n_dih_types;
    d->dih_params = s->dih_params.data();
    d->scaled14 = s->scaled14.data();
    d->isspa_type = s->isspa_type.data();
    d->n_isspa_types = s->n_isspa_types;
    d->rmax = s->rmax.data();
    d->n_g = s->n_g;
    d->n_e = s->n_e;
    d->n_f = s->n_f;
    d->g_table = s->g_table.data();
    d->e_table = s->e_table.data();
    d->f_table = s->f_table.data();
    d->g_r0 = s->g_r0; d->g_dr = s->g_dr;
    d->e_r0 = s->e_r0; d->e_dr = s->e_dr;
    d->f_r0 = s->f_r0; d->f_dr = s->f_dr;
    d->us_on = s->us_on;
    d->n_bias = (int)s->bias_list.size() / 2;
    d->bias_list = s->bias_list.data();
    d->us_k = s->us_k;
    d->us_x0 = s->us_x0;
    d->n_mc = s->n_mc;
    d->box = s->box;
    d->kT = s->kT;
    d->dt = s->dt;
    d->pnu = s->pnu;
    d->seed = s->seed;
    return ISSPA_OK;
}

void isspa_system_free(isspa_host_system *s) { delete s; }

// The sections isspa_read_isspatop reads, in the layout of the reference's
// .isspatop files (isspa_class.cpp:45-178; written there by
// scripts/isspa_prmtop/write_isspa_prmtop.py:202-273).  ISSPA_FORCES is written
// as the linear values the CUDA reader uses (isspa_class.cpp:155-170), not the
// logarithm that script stores.  Radii are r0 + i dr; values carry 9
// significant digits, so every float table entry reads back exactly.
int isspa_write_isspatop(const isspa_system_desc *d, const char *path, const char *title) {
    if (!d || !path || d->n_atoms <= 0 || d->n_isspa_types <= 0 || !d->isspa_type || !d->rmax || !d->g_table ||
        !d->e_table || !d->f_table || d->n_g < 2 || d->n_e < 2 || d->n_f < 2)
        return ISSPA_ERR_ARG;
    const int N = d->n_atoms, nt = d->n_isspa_types;
    for (int i = 0; i < N; ++i)
        if (d->isspa_type[i] < 0 || d->isspa_type[i] >= nt) return ISSPA_ERR_ARG;
    std::FILE *f = std::fopen(path, "w");
    if (!f) return ISSPA_ERR_IO;
    std::fprintf(f, "%%VERSION \n%%FLAG TITLE\n%%FORMAT(20a4)\n%.80s\n", title ? title : "");
    std::fprintf(f, "%%FLAG POINTERS\n%%FORMAT(10I8)\n%8d%8d%8d%8d%8d\n", N, nt, d->n_g, d->n_e, d->n_f);
    std::fprintf(f, "%%FLAG ISSPA_TYPE_INDEX\n%%FORMAT(10I8)\n");
    for (int i = 0; i < N; ++i)
        std::fprintf(f, "%8d%s", d->isspa_type[i] + 1, (i % 10 == 9 || i == N - 1) ? "\n" : "");
    std::fprintf(f, "%%FLAG ISSPA_RMAX\n%%FORMAT(5E16.8)\n");
    for (int t = 0; t < nt; ++t)
        std::fprintf(f, "%16.8e%s", (double)d->rmax[t], (t % 5 == 4 || t == nt - 1) ? "\n" : "");
    auto table = [&](const char *flag, int rows, const float *tab, float r0, float dr) {
        std::fprintf(f, "%%FLAG %s\n%%FORMAT(%dE16.8)\n", flag, nt + 1);
        for (int i = 0; i < rows; ++i) {
            std::fprintf(f, "%16.8e", (double)r0 + (double)i * (double)dr);
            for (int t = 0; t < nt; ++t) std::fprintf(f, "%16.8e", (double)tab[(size_t)t * rows + i]);
            std::fprintf(f, "\n");
        }
    };
    table("ISSPA_DENSITIES", d->n_g, d->g_table, d->g_r0, d->g_dr);
    table("ISSPA_EFIELD", d->n_e, d->e_table, d->e_r0, d->e_dr);
    table("ISSPA_FORCES", d->n_f, d->f_table, d->f_r0, d->f_dr);
    const bool ok = std::ferror(f) == 0;
    return (std::fclose(f) == 0 && ok) ? ISSPA_OK : ISSPA_ERR_IO;
}

}  // extern "C"

namespace isspa {

int host_system_from_desc(const isspa_system_desc &d, isspa_host_system &s) {
    if (d.n_atoms <= 0 || !d.pos || !d.vel || !d.lj_type || !d.nb_parm_index || !d.lj_ab ||
        !d.isspa_type || !d.rmax || !d.g_table || !d.e_table || !d.f_table || d.n_lj_types <= 0 ||
        d.n_isspa_types <= 0 || d.n_g < 2 || d.n_e < 2 || d.n_f < 2 || d.n_mc <= 0 || !(d.box > 0.f))
        return ISSPA_ERR_ARG;
    const int N = d.n_atoms;
    auto cp = [](auto *p, size_t n, auto &v) {
        v.assign(p, p + n);
    };
    s.n_atoms = N;
    cp(d.pos, 4 * (size_t)N, s.pos);
    cp(d.vel, 4 * (size_t)N, s.vel);
    if (d.raw_mass) cp(d.raw_mass, N, s.raw_mass);
    else {
        s.raw_mass.resize(N);
        for (int i = 0; i < N; ++i) s.raw_mass[i] = d.vel[4 * i + 3];
    }
    s.n_lj_types = d.n_lj_types;
    cp(d.lj_type, N, s.lj_type);
    cp(d.nb_parm_index, (size_t)d.n_lj_types * d.n_lj_types, s.nb_parm_index);
    cp(d.lj_ab, 2 * (size_t)(d.n_lj_types * (d.n_lj_types + 1) / 2), s.lj_ab);
    if (d.n_excl_cum) cp(d.n_excl_cum, N, s.n_excl_cum);
    else s.n_excl_cum.assign(N, 0);
    if (d.excl_len > 0 && d.excl_list) cp(d.excl_list, d.excl_len, s.excl_list);
    else s.excl_list.clear();
    // parameter tables whenever types are declared (a system may declare
    // types and have no terms of that kind); terms only when present
    if (d.n_bond_types < 0 || d.n_angle_types < 0 || d.n_dih_types < 0 || d.n_bonds < 0 || d.n_angles < 0 ||
        d.n_dihs < 0)
        return ISSPA_ERR_ARG;
    if ((d.n_bond_types > 0 && !d.bond_params) || (d.n_angle_types > 0 && !d.angle_params) ||
        (d.n_dih_types > 0 && (!d.dih_params || !d.scaled14)))
        return ISSPA_ERR_ARG;
    s.n_bond_types = d.n_bond_types;
    if (d.n_bond_types > 0) cp(d.bond_params, 2 * (size_t)d.n_bond_types, s.bond_params);
    if (d.n_bonds > 0) {
        if (!d.bond_atoms) return ISSPA_ERR_ARG;
        cp(d.bond_atoms, 3 * (size_t)d.n_bonds, s.bond_atoms);
    }
    s.n_angle_types = d.n_angle_types;
    if (d.n_angle_types > 0) cp(d.angle_params, 2 * (size_t)d.n_angle_types, s.angle_params);
    if (d.n_angles > 0) {
        if (!d.angle_atoms) return ISSPA_ERR_ARG;
        cp(d.angle_atoms, 4 * (size_t)d.n_angles, s.angle_atoms);
    }
    s.n_dih_types = d.n_dih_types;
    if (d.n_dih_types > 0) {
        cp(d.dih_params, 4 * (size_t)d.n_dih_types, s.dih_params);
        cp(d.scaled14, 2 * (size_t)d.n_dih_types, s.scaled14);
    }
    if (d.n_dihs > 0) {
        if (!d.dih_atoms || !d.dih_types) return ISSPA_ERR_ARG;
        cp(d.dih_atoms, 4 * (size_t)d.n_dihs, s.dih_atoms);
        cp(d.dih_types, d.n_dihs, s.dih_types);
    }
    s.have_isspa = true;
    cp(d.isspa_type, N, s.isspa_type);
    s.n_isspa_types = d.n_isspa_types;
    cp(d.rmax, d.n_isspa_types, s.rmax);
    s.n_g = d.n_g;
    s.n_e = d.n_e;
    s.n_f = d.n_f;
    cp(d.g_table, (size_t)d.n_isspa_types * d.n_g, s.g_table);
    cp(d.e_table, (size_t)d.n_isspa_types * d.n_e, s.e_table);
    cp(d.f_table, (size_t)d.n_isspa_types * d.n_f, s.f_table);
    s.g_r0 = d.g_r0; s.g_dr = d.g_dr;
    s.e_r0 = d.e_r0; s.e_dr = d.e_dr;
    s.f_r0 = d.f_r0; s.f_dr = d.f_dr;
    s.us_on = d.us_on;
    if (d.us_on) {
        if (d.n_bias <= 0 || !d.bias_list) return ISSPA_ERR_ARG;
        cp(d.bias_list, 2 * (size_t)d.n_bias, s.bias_list);
    }
    s.us_k = d.us_k;
    s.us_x0 = d.us_x0;
    s.n_mc = d.n_mc;
    s.box = d.box;
    s.kT = d.kT;
    s.dt = d.dt;
    s.pnu = d.pnu;
    s.seed = d.seed;
    // validation of what the kernels index
    const int nt = s.n_lj_types, ntt = nt * (nt + 1) / 2;
    for (int i = 0; i < N; ++i) {
        if (s.lj_type[i] < 0 || s.lj_type[i] >= nt) return ISSPA_ERR_ARG;
        if (s.isspa_type[i] < 0 || s.isspa_type[i] >= s.n_isspa_types) return ISSPA_ERR_ARG;
        if (!(s.vel[4 * i + 3] > 0.f)) return ISSPA_ERR_ARG;
    }
    for (int v : s.nb_parm_index) if (v < 0 || v >= ntt) return ISSPA_ERR_ARG;
    for (float r : s.rmax) if (!(r > 0.f)) return ISSPA_ERR_ARG;
    if (!(s.g_dr > 0.f && s.e_dr > 0.f && s.f_dr > 0.f)) return ISSPA_ERR_ARG;
    int prev = 0;
    for (int c : s.n_excl_cum) {
        if (c < prev || c > (int)s.excl_list.size()) return ISSPA_ERR_ARG;
        prev = c;
    }
    for (size_t b = 0; b < s.bond_atoms.size() / 3; ++b) {
        const int *a = &s.bond_atoms[3 * b];
        if (a[0] < 0 || a[0] >= N || a[1] < 0 || a[1] >= N || a[2] < 0 || a[2] >= s.n_bond_types) return ISSPA_ERR_ARG;
    }
    for (size_t b = 0; b < s.angle_atoms.size() / 4; ++b) {
        const int *a = &s.angle_atoms[4 * b];
        for (int k = 0; k < 3; ++k) if (a[k] < 0 || a[k] >= N) return ISSPA_ERR_ARG;
        if (a[3] < 0 || a[3] >= s.n_angle_types) return ISSPA_ERR_ARG;
    }
    for (size_t b = 0; b < s.dih_types.size(); ++b) {
        const int *a = &s.dih_atoms[4 * b];
        for (int k = 0; k < 4; ++k) if (std::abs(a[k]) >= N) return ISSPA_ERR_ARG;
        if (s.dih_types[b] < 0 || s.dih_types[b] >= s.n_dih_types) return ISSPA_ERR_ARG;
    }
    for (size_t b = 0; b < s.bias_list.size() / 2; ++b) {
        if (s.bias_list[2 * b] < 0 || s.bias_list[2 * b] >= N) return ISSPA_ERR_ARG;
        if (s.bias_list[2 * b + 1] != 0 && s.bias_list[2 * b + 1] != 1) return ISSPA_ERR_ARG;
    }
    return ISSPA_OK;
}

void init_velocities(isspa_host_system &s, uint64_t seed) {
    // Maxwell-Boltzmann draw at kT from Philox stream 2 (Box-Muller); the
    // reference draws from glibc rand() (atom_class.cpp:53-64, :158-173).
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int i = 0; i < s.n_atoms; ++i) {
        u32x4 o = philox4x32_10(u32x4{(uint32_t)i, 0u, 0u, 2u}, k0, k1);
        double u0 = u01_open0(o.x), u1 = u01(o.y), u2 = u01_open0(o.z), u3 = u01(o.w);
        double ra = std::sqrt(-2.0 * std::log(u0)), rb = std::sqrt(-2.0 * std::log(u2));
        double n[3] = {ra * std::cos(6.283185307179586 * u1), ra * std::sin(6.283185307179586 * u1),
                       rb * std::cos(6.283185307179586 * u3)};
        double sd = std::sqrt((double)s.kT / s.vel[4 * i + 3]);
        for (int k = 0; k < 3; ++k) s.vel[4 * i + k] = (float)(n[k] * sd);
    }
}

}  // namespace isspa
