// config.cpp - YAML parameters of the hot path (host side).
//
// Mirrors the reference's configuration layer for the hot-path sections:
// YAML defaults merged with user overrides (src/freeform/main.cpp:97-106,
// src/utils/yaml.cpp:4-42), unit-bearing values evaluated as arithmetic over
// unit symbols (src/utils/units.cpp:12-52, constants from
// include/xmd/utils/units.h:11-62) and the per-section readers of
// src/freeform/params.cpp:43-197, src/types/amino_acid.cpp:83-150 and
// src/forces/primitives/lj_variants.cpp:8-63.
#include "config.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>
#include <stdexcept>

namespace xmdg {

// ---------------------------------------------------------------- YAML --

const YNode *YNode::get(const std::string &key) const {
    if (kind != Map) return nullptr;
    for (auto &kv : map)
        if (kv.first == key) return &kv.second;
    return nullptr;
}
YNode *YNode::get_mut(const std::string &key) {
    if (kind != Map) return nullptr;
    for (auto &kv : map)
        if (kv.first == key) return &kv.second;
    return nullptr;
}

namespace {

struct Line {
    int no;          // 1-based line number
    int indent;      // leading spaces
    std::string raw; // full line without newline
    std::string body;// content after indentation, comment stripped, right-trimmed
};

std::string rtrim(std::string s) {
    while (!s.empty() && (s.back() == ' ' || s.back() == '\t' || s.back() == '\r')) s.pop_back();
    return s;
}
std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

std::string strip_comment(const std::string &s) {
    char q = 0;
    for (size_t i = 0; i < s.size(); ++i) {
        char c = s[i];
        if (q) {
            if (c == q) q = 0;
        } else if (c == '"' || c == '\'') {
            if (i == 0 || s[i - 1] == ' ' || s[i - 1] == ':' || s[i - 1] == '[' || s[i - 1] == ',') q = c;
        } else if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) {
            return s.substr(0, i);
        }
    }
    return s;
}

[[noreturn]] void fail(int line, const std::string &msg) {
    throw std::runtime_error("YAML line " + std::to_string(line) + ": " + msg);
}

std::string unquote(const std::string &v, int line) {
    if (v.size() >= 2 && (v[0] == '"' || v[0] == '\'')) {
        if (v.back() != v[0]) fail(line, "unterminated quoted scalar");
        std::string out;
        for (size_t i = 1; i + 1 < v.size(); ++i) {
            if (v[0] == '"' && v[i] == '\\' && i + 2 < v.size()) {
                char n = v[++i];
                out += n == 'n' ? '\n' : n == 't' ? '\t' : n;
            } else if (v[0] == '\'' && v[i] == '\'' && i + 2 < v.size() && v[i + 1] == '\'') {
                out += '\''; ++i;
            } else {
                out += v[i];
            }
        }
        return out;
    }
    return v;
}

// split "key: value" at the first ": " (or trailing ':') outside quotes
bool split_key(const std::string &body, std::string &key, std::string &val) {
    char q = 0;
    for (size_t i = 0; i < body.size(); ++i) {
        char c = body[i];
        if (q) { if (c == q) q = 0; continue; }
        if ((c == '"' || c == '\'') && i == 0) { q = c; continue; }
        if (c == ':' && (i + 1 == body.size() || body[i + 1] == ' ')) {
            key = trim(body.substr(0, i));
            val = trim(body.substr(i + 1));
            return true;
        }
    }
    return false;
}

YNode scalar_node(const std::string &v, int line) {
    YNode n;
    std::string t = trim(v);
    if (t.empty() || t == "~" || t == "null") { n.kind = YNode::Null; return n; }
    if (t[0] == '[') {
        if (t.back() != ']') fail(line, "flow sequence must close on the same line");
        n.kind = YNode::Seq;
        std::string inner = trim(t.substr(1, t.size() - 2));
        if (inner.empty()) return n;
        std::string cur;
        char q = 0;
        for (char c : inner) {
            if (q) { cur += c; if (c == q) q = 0; continue; }
            if (c == '"' || c == '\'') { q = c; cur += c; continue; }
            if (c == ',') { n.seq.push_back(scalar_node(cur, line)); cur.clear(); continue; }
            cur += c;
        }
        n.seq.push_back(scalar_node(cur, line));
        return n;
    }
    if (t[0] == '{') fail(line, "flow mappings are not supported");
    n.kind = YNode::Scalar;
    n.scalar = unquote(t, line);
    return n;
}

struct Parser {
    std::vector<Line> lines;
    size_t pos = 0;

    void skip_blank() {
        while (pos < lines.size() && lines[pos].body.empty()) ++pos;
    }

    YNode block(int indent) {
        skip_blank();
        YNode node;
        if (pos >= lines.size()) return node;
        const Line &first = lines[pos];
        if (first.indent < indent) return node;
        int my_indent = first.indent;
        bool is_seq = first.body.rfind("- ", 0) == 0 || first.body == "-";
        node.kind = is_seq ? YNode::Seq : YNode::Map;
        while (true) {
            skip_blank();
            if (pos >= lines.size()) break;
            const Line &ln = lines[pos];
            if (ln.indent < my_indent) break;
            if (ln.indent > my_indent) fail(ln.no, "unexpected indentation");
            if (is_seq) {
                if (!(ln.body.rfind("- ", 0) == 0 || ln.body == "-")) fail(ln.no, "expected '- ' item");
                std::string item = ln.body.size() > 1 ? trim(ln.body.substr(2)) : "";
                ++pos;
                std::string k, v;
                if (!item.empty() && split_key(item, k, v))
                    fail(ln.no, "mappings inside block sequences are not supported");
                if (item.empty()) node.seq.push_back(block(my_indent + 1));
                else node.seq.push_back(scalar_node(item, ln.no));
                continue;
            }
            std::string key, val;
            if (!split_key(ln.body, key, val)) fail(ln.no, "expected 'key: value'");
            key = unquote(key, ln.no);
            ++pos;
            YNode child;
            if (val == "|" || val == "|-" || val == "|+") {
                child.kind = YNode::Scalar;
                int content_indent = -1;
                std::vector<std::string> parts;
                while (pos < lines.size()) {
                    const Line &bl = lines[pos];
                    std::string rt = rtrim(bl.raw);
                    if (rt.empty()) { parts.push_back(""); ++pos; continue; }
                    int ind = 0;
                    while (ind < (int)bl.raw.size() && bl.raw[ind] == ' ') ++ind;
                    if (ind <= my_indent) break;
                    if (content_indent < 0) content_indent = ind;
                    if (ind < content_indent) break;
                    parts.push_back(rt.substr(content_indent));
                    ++pos;
                }
                while (!parts.empty() && parts.back().empty()) parts.pop_back();
                std::string text;
                for (size_t i = 0; i < parts.size(); ++i) {
                    if (i) text += '\n';
                    text += parts[i];
                }
                if (val == "|" && !text.empty()) text += '\n';
                child.scalar = text;
            } else if (val.empty()) {
                skip_blank();
                if (pos < lines.size() && lines[pos].indent > my_indent) child = block(my_indent + 1);
                else if (pos < lines.size() && lines[pos].indent == my_indent &&
                         lines[pos].body.rfind("- ", 0) == 0)
                    child = block(my_indent);
                else child.kind = YNode::Null;
            } else {
                child = scalar_node(val, ln.no);
            }
            bool replaced = false;
            for (auto &kv : node.map)
                if (kv.first == key) { kv.second = child; replaced = true; }
            if (!replaced) node.map.emplace_back(key, child);
        }
        return node;
    }
};

}  // namespace

YNode parse_yaml(const std::string &text) {
    Parser ps;
    std::istringstream in(text);
    std::string raw;
    int no = 0;
    while (std::getline(in, raw)) {
        ++no;
        if (!raw.empty() && raw.back() == '\r') raw.pop_back();
        for (char c : raw) {
            if (c == '\t') throw std::runtime_error("YAML line " + std::to_string(no) + ": tab character");
            if (c != ' ') break;
        }
        Line ln;
        ln.no = no;
        ln.raw = raw;
        int ind = 0;
        while (ind < (int)raw.size() && raw[ind] == ' ') ++ind;
        ln.indent = ind;
        std::string b = rtrim(strip_comment(raw.substr(ind)));
        if (b == "---" || b == "...") b.clear();
        ln.body = b;
        ps.lines.push_back(ln);
    }
    ps.skip_blank();
    if (ps.pos >= ps.lines.size()) return YNode();
    YNode root = ps.block(0);
    ps.skip_blank();
    if (ps.pos < ps.lines.size()) fail(ps.lines[ps.pos].no, "unexpected content");
    return root;
}

YNode merge_yaml(const YNode &defaults, const YNode &overrides) {
    if (overrides.kind != YNode::Map) return overrides.kind == YNode::Null ? defaults : overrides;
    if (defaults.kind != YNode::Map) return overrides;
    YNode out;
    out.kind = YNode::Map;
    for (auto &kv : defaults.map) {
        const YNode *o = overrides.get(kv.first);
        out.map.emplace_back(kv.first, o ? merge_yaml(kv.second, *o) : kv.second);
    }
    for (auto &kv : overrides.map)
        if (!defaults.get(kv.first)) out.map.push_back(kv);
    return out;
}

// --------------------------------------------------------------- units --

double unit_value(const std::string &name) {
    // include/xmd/utils/units.h:11-62, evaluated in double like `Unit`
    static const std::map<std::string, double> table = [] {
        const double f77unit = 1.0, angstrom = f77unit / 5.0, nanometer = 10.0 * angstrom,
                     meter = nanometer * 1.0e9;
        const double nanosecond = 1.0, tau = 1.0 * nanosecond, microsecond = nanosecond * 1.0e3,
                     millisecond = nanosecond * 1.0e6, second = nanosecond * 1.0e9;
        const double atom = 1.0, mol = 6.02214076e23 / atom;
        const double eps = 1.0, kcal = eps * mol / 1.57824959, Joule = kcal / 4184.0;
        const double eps_kB = 1.0, kB = eps / eps_kB, Kelvin = 1.380649e-23 * Joule / kB;
        const double kg = Joule * second * second / (meter * meter), amu = kg * 0.99999999965e-3 / mol;
        const double f77mass = eps * tau * tau / (f77unit * f77unit);
        const double echarge = 1.0, Coulomb = echarge / 1.602176634e-19, Ampere = Coulomb / second;
        const double cspeed = 299792458.0 * meter / second;
        const double Henry = kg * meter * meter / (second * second * Ampere * Ampere);
        const double mu_0 = 1.25663706212e-6 * Henry / meter;
        const double eps_0 = 1.0 / (mu_0 * cspeed * cspeed);
        const double rad = 1.0, deg = (2.0 * M_PI / 360.0) * rad;
        return std::map<std::string, double>{
            {"f77unit", f77unit}, {"A", angstrom}, {"nm", nanometer}, {"m", meter},
            {"ns", nanosecond}, {"tau", tau}, {"micros", microsecond}, {"ms", millisecond},
            {"s", second}, {"atom", atom}, {"mol", mol}, {"eps", eps}, {"kcal", kcal},
            {"J", Joule}, {"kB", kB}, {"K", Kelvin}, {"kg", kg}, {"amu", amu},
            {"f77mass", f77mass}, {"e", echarge}, {"C", Coulomb}, {"Amp", Ampere},
            {"c", cspeed}, {"H", Henry}, {"mu_0", mu_0}, {"eps_0", eps_0}, {"rad", rad},
            {"deg", deg}};
    }();
    auto it = table.find(name);
    if (it == table.end()) throw std::runtime_error("unknown unit symbol '" + name + "'");
    return it->second;
}

namespace {
// arithmetic over numbers and unit symbols: + - * / ** ^ ( ) and unary signs
struct Expr {
    const std::string &s;
    size_t i = 0;
    explicit Expr(const std::string &str) : s(str) {}
    void ws() { while (i < s.size() && std::isspace((unsigned char)s[i])) ++i; }
    [[noreturn]] void bad(const char *m) {
        throw std::runtime_error(std::string("bad quantity '") + s + "': " + m);
    }
    double primary() {
        ws();
        if (i >= s.size()) bad("unexpected end");
        char c = s[i];
        if (c == '(') {
            ++i;
            double v = sum();
            ws();
            if (i >= s.size() || s[i] != ')') bad("missing ')'");
            ++i;
            return v;
        }
        if (std::isdigit((unsigned char)c) || c == '.') {
            const char *b = s.c_str() + i;
            char *e = nullptr;
            double v = std::strtod(b, &e);
            if (e == b) bad("bad number");
            i += (size_t)(e - b);
            return v;
        }
        if (std::isalpha((unsigned char)c) || c == '_') {
            size_t b = i;
            while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_')) ++i;
            return unit_value(s.substr(b, i - b));
        }
        bad("unexpected character");
    }
    double unary() {
        ws();
        if (i < s.size() && s[i] == '-') { ++i; return -unary(); }
        if (i < s.size() && s[i] == '+') { ++i; return unary(); }
        return power();
    }
    double power() {
        double b = primary();
        ws();
        if (i + 1 < s.size() && s[i] == '*' && s[i + 1] == '*') { i += 2; return std::pow(b, unary()); }
        if (i < s.size() && s[i] == '^') { ++i; return std::pow(b, unary()); }
        return b;
    }
    double product() {
        double v = unary();
        while (true) {
            ws();
            if (i < s.size() && s[i] == '*' && !(i + 1 < s.size() && s[i + 1] == '*')) { ++i; v *= unary(); }
            else if (i < s.size() && s[i] == '/') { ++i; v /= unary(); }
            else return v;
        }
    }
    double sum() {
        double v = product();
        while (true) {
            ws();
            if (i < s.size() && s[i] == '+') { ++i; v += product(); }
            else if (i < s.size() && s[i] == '-') { ++i; v -= product(); }
            else return v;
        }
    }
    double all() {
        double v = sum();
        ws();
        if (i != s.size()) bad("trailing characters");
        return v;
    }
};
}  // namespace

double parse_quantity(const std::string &str, double def_unit) {
    std::string s = trim(str);
    auto sp = s.find(' ');
    if (sp == std::string::npos) {
        Expr e(s);
        return e.all() * def_unit;
    }
    std::string mag = s.substr(0, sp), unit = trim(s.substr(sp + 1));
    Expr em(mag), eu(unit);
    return em.all() * eu.all();
}

// ------------------------------------------------------------ resolver --

namespace {
const char *kAA[XMD_NUM_AA] = {"ALA", "ARG", "ASN", "ASP", "CYS", "GLU", "GLN",
                               "GLY", "HIS", "ILE", "LEU", "LYS", "MET", "PHE",
                               "PRO", "SER", "THR", "TRP", "TYR", "VAL"};

int aa_index(const std::string &name) {
    for (int k = 0; k < XMD_NUM_AA; ++k)
        if (name == kAA[k]) return k;
    throw std::runtime_error("unknown amino acid '" + name + "'");
}

const YNode &need(const YNode &n, const std::string &key, const std::string &where) {
    const YNode *c = n.get(key);
    if (!c || c->kind == YNode::Null) throw std::runtime_error("missing key '" + where + key + "'");
    return *c;
}
const YNode &section(const YNode &root, const std::string &key) { return need(root, key, ""); }
std::string sval(const YNode &n, const std::string &key, const std::string &where) {
    const YNode &c = need(n, key, where);
    if (c.kind != YNode::Scalar) throw std::runtime_error("key '" + where + key + "' is not a scalar");
    return c.scalar;
}
double qval(const YNode &n, const std::string &key, const std::string &where, double def_unit = 1.0) {
    try {
        return parse_quantity(sval(n, key, where), def_unit);
    } catch (std::runtime_error &e) {
        throw std::runtime_error("'" + where + key + "': " + e.what());
    }
}
bool bval(const YNode &n, const std::string &key, const std::string &where) {
    std::string v = sval(n, key, where);
    for (auto &c : v) c = (char)std::tolower((unsigned char)c);
    if (v == "true" || v == "yes" || v == "on" || v == "y") return true;
    if (v == "false" || v == "no" || v == "off" || v == "n") return false;
    throw std::runtime_error("key '" + where + key + "' is not a boolean");
}
bool enabled(const YNode &root, const std::string &sec) {
    const YNode *s = root.get(sec);
    if (!s) return false;
    return bval(*s, "enabled", sec + ": ");
}

// csv_file of src/files/csv.cpp: header row, then records
std::vector<std::vector<std::string>> read_csv(const std::string &text) {
    std::vector<std::vector<std::string>> rows;
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        line = trim(line);
        if (line.empty()) continue;
        std::vector<std::string> f;
        std::string cur;
        for (char c : line) {
            if (c == ',') { f.push_back(trim(cur)); cur.clear(); }
            else cur += c;
        }
        f.push_back(trim(cur));
        rows.push_back(f);
    }
    return rows;
}

void read_ss_table(const std::string &csv, double def_unit, double *out) {
    auto rows = read_csv(csv);
    if (rows.empty()) return;
    auto &hdr = rows[0];
    std::vector<int> col(hdr.size(), -1);
    int type_col = -1;
    for (size_t k = 0; k < hdr.size(); ++k) {
        if (hdr[k] == "type") type_col = (int)k;
        else if (!hdr[k].empty()) col[k] = aa_index(hdr[k]);
    }
    if (type_col < 0) throw std::runtime_error("per-pair table has no 'type' column");
    for (size_t r = 1; r < rows.size(); ++r) {
        int a1 = aa_index(rows[r][type_col]);
        for (size_t k = 0; k < rows[r].size() && k < hdr.size(); ++k) {
            if (col[k] < 0 || rows[r][k].empty()) continue;
            // lj_variants.cpp:39-43: ss_idx = NUM_AA*aa1 + aa2
            out[XMD_NUM_AA * a1 + col[k]] = parse_quantity(rows[r][k], def_unit);
        }
    }
}
// Heuristic coefficient tables (freeform/params.cpp:69-83, 101-118): two
// residue-class columns (G, P, anything else = X), then the coefficients by
// position.  The shipped header names fewer columns than the rows hold
// (a0..a5 for 7 angle coefficients; no constant column for the dihedral's
// 6), so the coefficients are read in row order: a0..a6 and c0..c5, the
// orders eval_heurestic_angle_forces / eval_heurestic_dihedral_forces use.
int heur_class(const std::string &s) {
    if (s.empty()) throw std::runtime_error("empty residue class in a heuristic table");
    return s[0] == 'G' ? 0 : (s[0] == 'P' ? 1 : 2);
}

void read_heur_table(const std::string &csv, int ncoef, double *out, const std::string &where) {
    auto rows = read_csv(csv);
    for (size_t r = 1; r < rows.size(); ++r) {
        const auto &f = rows[r];
        if (f.size() < 2) throw std::runtime_error(where + "short row");
        const int type = 3 * heur_class(f[0]) + heur_class(f[1]);
        int k = 0;
        for (size_t c = 2; c < f.size(); ++c) {
            if (f[c].empty()) continue;
            if (k == ncoef) throw std::runtime_error(where + "too many coefficients in a row");
            out[type * ncoef + k++] = parse_quantity(f[c], 1.0);
        }
        if (k != ncoef) throw std::runtime_error(where + "too few coefficients in a row");
    }
}
}  // namespace

void resolve_params(const YNode &root, xmd_params *o) {
    std::memset(o, 0, sizeof *o);
    const double A = unit_value("A"), eps = unit_value("eps");
    // general: params.cpp:7-11
    {
        const YNode &g = section(root, "general");
        o->total_time = qval(g, "total time", "general: ");
        std::string sd = sval(g, "seed", "general: ");
        o->seed = std::strtoull(sd.c_str(), nullptr, 10);
    }
    // langevin / integrator: params.cpp:43-53
    {
        const YNode &l = section(root, "langevin");
        o->langevin_on = bval(l, "enabled", "langevin: ");
        o->gamma_factor = qval(l, "gamma factor", "langevin: ");
        o->temperature = qval(l, "temperature", "langevin: ");
        const YNode &in = section(root, "integrator");
        o->dt = qval(in, "dt", "integrator: ");
    }
    // neighbor list: params.cpp:54-56 (+ additive cutoff/skin keys)
    {
        const YNode &nl = section(root, "neighbor list");
        o->pad_factor = qval(nl, "pad factor", "neighbor list: ");
        o->nl_cutoff = nl.get("cutoff") ? qval(nl, "cutoff", "neighbor list: ", A) : 0.0;
        o->nl_skin = nl.get("skin") ? qval(nl, "skin", "neighbor list: ", A) : 0.0;
    }
    o->on[XMD_TERM_TETHER] = enabled(root, "tether forces");
    {
        const YNode &t = section(root, "tether forces");
        o->tether_H1 = qval(t, "H1", "tether forces: ");
        o->tether_H2 = qval(t, "H2", "tether forces: ");
        o->tether_def_length = qval(t, "default bond length", "tether forces: ");
    }
    o->on[XMD_TERM_NAT_ANG] = enabled(root, "native angles");
    o->nat_ang_k = qval(section(root, "native angles"), "k", "native angles: ");
    o->on[XMD_TERM_CND] = enabled(root, "complex native dihedrals");
    o->cnd_CDA = qval(section(root, "complex native dihedrals"), "CDA", "complex native dihedrals: ");
    o->cnd_CDB = qval(section(root, "complex native dihedrals"), "CDB", "complex native dihedrals: ");
    o->on[XMD_TERM_SND] = enabled(root, "simple native dihedrals");
    o->snd_CDH = qval(section(root, "simple native dihedrals"), "CDH", "simple native dihedrals: ");
    o->on[XMD_TERM_GO] = enabled(root, "native contacts");
    {
        const YNode &nc = section(root, "native contacts");
        o->go_depth = qval(nc, "lj depth", "native contacts: ");
        o->go_active_threshold = qval(nc, "active threshold", "native contacts: ");
    }
    o->on[XMD_TERM_PAULI] = enabled(root, "Pauli exclusion");
    o->pauli_r_excl = qval(section(root, "Pauli exclusion"), "r_excl", "Pauli exclusion: ");
    o->pauli_depth = qval(section(root, "Pauli exclusion"), "depth", "Pauli exclusion: ");
    o->on[XMD_TERM_CONST_ES] = enabled(root, "const ES");
    o->const_es_screen_dist = qval(section(root, "const ES"), "screening distance", "const ES: ");
    o->const_es_permittivity = qval(section(root, "const ES"), "permittivity", "const ES: ");
    o->on[XMD_TERM_REL_ES] = enabled(root, "relative ES");
    o->rel_es_screen_dist = qval(section(root, "relative ES"), "screening distance", "relative ES: ");
    o->rel_es_factor = qval(section(root, "relative ES"), "factor", "relative ES: ");
    o->on[XMD_TERM_CHIR] = enabled(root, "chirality");
    o->chir_e_chi = qval(section(root, "chirality"), "e_chi", "chirality: ");
    o->on[XMD_TERM_NAT_SS] = enabled(root, "native ssbonds");
    o->nat_ss_H1 = qval(section(root, "native ssbonds"), "H1", "native ssbonds: ");
    o->nat_ss_dist = qval(section(root, "native ssbonds"), "equilibrium dist", "native ssbonds: ");
    o->on[XMD_TERM_HEUR_ANG] = enabled(root, "heurestic angles");
    read_heur_table(sval(section(root, "heurestic angles"), "coefficients", "heurestic angles: "), 7,
                    &o->heur_ang_coeffs[0][0], "heurestic angles: ");
    o->on[XMD_TERM_HEUR_DIH] = enabled(root, "heurestic dihedrals");
    read_heur_table(sval(section(root, "heurestic dihedrals"), "coefficients", "heurestic dihedrals: "), 6,
                    &o->heur_dih_coeffs[0][0], "heurestic dihedrals: ");
    o->on[XMD_TERM_VEL_AFM] = enabled(root, "velocity AFM");
    o->vel_afm_H1 = qval(section(root, "velocity AFM"), "H1", "velocity AFM: ");
    o->vel_afm_H2 = qval(section(root, "velocity AFM"), "H2", "velocity AFM: ");
    o->on[XMD_TERM_FORCE_AFM] = enabled(root, "force AFM");
    {
        // pid_params (freeform/params.cpp:132-158); an unknown lambda
        // version is cosine (main.cpp:765-767)
        const YNode &q = section(root, "pseudo-improper dihedral potential");
        const std::string w = "pseudo-improper dihedral potential: ";
        o->on[XMD_TERM_PID] = enabled(root, "pseudo-improper dihedral potential");
        o->pid_lambda = sval(q, "lambda version", w) == "algebraic" ? 1 : 0;
        const YNode &bp = need(q, "bb+", w), &bm = need(q, "bb-", w), &ss = need(q, "ss", w);
        const char *keys[4] = {"alpha", "psi_0", "r_min", "depth"};
        for (int k = 0; k < 4; ++k) {
            o->pid_bbp[k] = qval(bp, keys[k], w + "bb+: ");
            o->pid_bbm[k] = qval(bm, keys[k], w + "bb-: ");
        }
        o->pid_ss[0] = qval(ss, "alpha", w + "ss: ");
        o->pid_ss[1] = qval(ss, "psi_0", w + "ss: ");
    }
    o->on[XMD_TERM_SOLID_WALL] = enabled(root, "solid walls");
    o->solid_wall_depth = qval(section(root, "solid walls"), "depth", "solid walls: ");
    o->solid_wall_cutoff = qval(section(root, "solid walls"), "cutoff", "solid walls: ");
    {
        const YNode &w = section(root, "LJ attractive walls");
        const std::string ws = "LJ attractive walls: ";
        o->on[XMD_TERM_LJ_WALL] = enabled(root, "LJ attractive walls");
        o->lj_wall_min_dist = qval(w, "wall min dist", ws);
        o->lj_wall_breaking_factor = qval(w, "breaking factor", ws);
        o->lj_wall_phase_duration = qval(w, "phase duration", ws);
        o->lj_wall_depth = qval(w, "depth", ws);
    }
    o->on[XMD_TERM_QA] = enabled(root, "quasi-adiabatic potential");
    {
        const YNode &q = section(root, "quasi-adiabatic potential");
        const std::string w = "quasi-adiabatic potential: ";
        o->qa_phase_duration = qval(q, "phase duration", w);
        o->qa_breaking_factor = qval(q, "breaking factor", w);
        o->qa_min_cos_hr = qval(q, "min |cos(h, r)|", w);
        o->qa_min_cos_hh = qval(q, "min |cos(h, h)| for bb", w);
        o->qa_max_cos_nr = qval(q, "max cos(n, r)", w);
    }
    // lj force variants: lj_variants.cpp:8-63
    {
        const YNode &lv = section(root, "lj force variants");
        const std::string w = "lj force variants: ";
        const YNode &bb = need(lv, "bb", w), &bs = need(lv, "bs", w), &ss = need(lv, "ss", w);
        o->lj_bb_r_min = qval(bb, "r_min", w + "bb: ");
        o->lj_bb_depth = qval(bb, "depth", w + "bb: ");
        o->lj_bs_r_min = qval(bs, "r_min", w + "bs: ");
        o->lj_bs_depth = qval(bs, "depth", w + "bs: ");
        if (const YNode *def = ss.get("default")) {
            if (def->get("r_max")) {
                double v = qval(*def, "r_max", w + "ss: default: ");
                for (int k = 0; k < XMD_NUM_SS; ++k) o->ss_r_max[k] = v;
            }
            if (def->get("depth")) {
                double v = qval(*def, "depth", w + "ss: default: ");
                for (int k = 0; k < XMD_NUM_SS; ++k) o->ss_depth[k] = v;
            }
        }
        if (const YNode *pp = ss.get("per pair")) {
            if (const YNode *t = pp->get("r_max"); t && t->kind == YNode::Scalar)
                read_ss_table(t->scalar, A, o->ss_r_max);
            if (const YNode *t = pp->get("depth"); t && t->kind == YNode::Scalar)
                read_ss_table(t->scalar, eps, o->ss_depth);
        }
        o->ss_sinking = bval(ss, "use sinking variant", w + "ss: ");
    }
    // amino acid data: amino_acid.cpp:83-150
    {
        const YNode &ad = section(root, "amino acid data");
        if (ad.get("from file"))
            throw std::runtime_error("'amino acid data: from file' is not supported; inline the table");
        const YNode &aas = need(ad, "amino acids", "amino acid data: ");
        for (auto &kv : aas.map) {
            int a = aa_index(kv.first);
            const YNode &d = kv.second;
            o->polarization[a] = 0;
            if (const YNode *pz = d.get("polarization"); pz && pz->kind == YNode::Scalar) {
                if (pz->scalar == "polar") o->polarization[a] = 1;
                else if (pz->scalar == "hydrophobic") o->polarization[a] = 2;
            }
            o->charge[a] = 0.0;
            if (const YNode *ch = d.get("charge"); ch && ch->kind == YNode::Scalar)
                o->charge[a] = parse_quantity(ch->scalar, unit_value("e"));
            for (int k = 0; k < 4; ++k) o->limits[a][k] = 0;
            if (const YNode *cl = d.get("contact limits"); cl && cl->kind == YNode::Map) {
                for (auto &lk : cl->map) {
                    int v = std::atoi(lk.second.scalar.c_str());
                    if (lk.first == "back") o->limits[a][0] = v;
                    else if (lk.first == "side (all)") o->limits[a][1] = v;
                    else if (lk.first == "side (polar)") o->limits[a][2] = v;
                    else if (lk.first == "side (hydrophobic)") o->limits[a][3] = v;
                }
            }
        }
    }
    // engine-only section
    o->precision = XMD_PREC_FP64;
    o->nl_capacity = 64;
    o->nl_grow = 1;
    o->device = 0;
    o->nl_build = XMD_NL_BUILD_AUTO;
    if (const YNode *en = root.get("engine")) {
        if (const YNode *nb = en->get("nl build"); nb && nb->kind == YNode::Scalar) {
            if (nb->scalar == "auto") o->nl_build = XMD_NL_BUILD_AUTO;
            else if (nb->scalar == "cell") o->nl_build = XMD_NL_BUILD_CELL;
            else if (nb->scalar == "tile") o->nl_build = XMD_NL_BUILD_TILE;
            else throw std::runtime_error("engine: nl build must be 'auto', 'cell' or 'tile'");
        }
        if (en->get("nl grow")) o->nl_grow = bval(*en, "nl grow", "engine: ");
        if (const YNode *dv = en->get("device"); dv && dv->kind == YNode::Scalar) {
            o->device = std::atoi(dv->scalar.c_str());
            if (o->device < 0) throw std::runtime_error("engine: device must be >= 0");
        }
        if (const YNode *nc = en->get("nl capacity"); nc && nc->kind == YNode::Scalar) {
            o->nl_capacity = std::atoi(nc->scalar.c_str());
            if (o->nl_capacity < 1) throw std::runtime_error("engine: nl capacity must be >= 1");
        }
        if (const YNode *pr = en->get("precision"); pr && pr->kind == YNode::Scalar) {
            if (pr->scalar == "fp64") o->precision = XMD_PREC_FP64;
            else if (pr->scalar == "mixed") o->precision = XMD_PREC_MIXED;
            else throw std::runtime_error("engine: precision must be 'fp64' or 'mixed'");
        }
    }
}

void params_from_yaml(const std::string &overrides_text, xmd_params *out) {
    YNode defaults = parse_yaml(defaults_yaml_text());
    YNode over = parse_yaml(overrides_text);
    YNode merged = merge_yaml(defaults, over);
    resolve_params(merged, out);
}

}  // namespace xmdg
