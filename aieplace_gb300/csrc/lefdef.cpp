// LEF/DEF ingest and DEF write-back for the placement library (host code).
//
// Replaces the reference host's DataBase ingest (vck5000/host/src/
// DataBase.cpp:42-96 readLEF / readDEF through Limbo's parsers, and the
// callbacks that keep data, :340-416: lef_macro_cbk, set_def_unit,
// set_def_design, set_def_diearea, add_def_component, add_def_pin,
// add_def_net) and DataBase::writeDEF (:538-655).  Only the subset those
// callbacks consume is interpreted -- LEF MACRO SIZE; DEF DESIGN, UNITS
// DISTANCE MICRONS, DIEAREA, COMPONENTS, PINS (first LAYER rectangle,
// placement, direction) and NETS (component and IO pin connections);
// everything else is skipped by the block structure of the two formats.
//
// Node order of the netlist view: DEF components in file order, then DEF IO
// pins in file order.  Components placed FIXED or COVER are fixed nodes;
// IO pins are fixed zero-area nodes that carry pins only (the reference
// leaves them out of the density map, AIEplace.cpp:937-958).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include <dirent.h>

#include "../../include/aieplace.h"

namespace {

thread_local std::string g_last_error;

struct Component {
    std::string name, model, orient;
    int status;  // 0 unplaced, 1 placed, 2 fixed, 3 cover
    double x, y;
};

struct IoPin {
    std::string name, net, direction, use, layer, orient;
    int status;  // as Component
    bool has_rect;
    long long rect[4];
    double x, y;
};

struct NetConn {
    int node;          // netlist node index
    std::string pin;   // component pin name ("PIN" connections: empty)
};

struct Net {
    std::string name;
    std::vector<NetConn> conns;
};

}  // namespace

struct ap_design {
    std::string design_name, def_version;
    int units = 1000;
    bool has_die = false;
    double die[4] = {0, 0, 0, 0};
    std::unordered_map<std::string, std::pair<double, double>> macros;  // LEF SIZE (microns)
    std::vector<Component> comps;
    std::vector<IoPin> pins;
    std::vector<Net> nets;
    int size_mode = AP_LEF_SIZE_DBU;
    // netlist view
    std::vector<int32_t> net_ptr, pin_node;
    std::vector<float> w, h, x, y;
    std::vector<uint8_t> fixed;
};

namespace {

// ---- tokenizer ---------------------------------------------------------------
// Whitespace-separated tokens; '(' ')' ';' are tokens of their own even when
// glued to a neighbour; "quoted strings" are one token; '#' starts a comment
// to the end of the line.
struct Lexer {
    std::string src, file;
    size_t pos = 0;
    int line = 1;
    std::string tok;
    int tok_line = 0;

    bool next() {
        for (;;) {
            while (pos < src.size() && std::isspace((unsigned char)src[pos])) {
                if (src[pos] == '\n') ++line;
                ++pos;
            }
            if (pos >= src.size()) {
                tok.clear();
                return false;
            }
            if (src[pos] == '#') {
                while (pos < src.size() && src[pos] != '\n') ++pos;
                continue;
            }
            break;
        }
        tok_line = line;
        const char c = src[pos];
        if (c == '(' || c == ')' || c == ';') {
            tok.assign(1, c);
            ++pos;
            return true;
        }
        if (c == '"') {
            size_t e = pos + 1;
            while (e < src.size() && src[e] != '"') {
                if (src[e] == '\n') ++line;
                ++e;
            }
            tok = src.substr(pos, e + 1 - pos);
            pos = e < src.size() ? e + 1 : e;
            return true;
        }
        size_t e = pos;
        while (e < src.size() && !std::isspace((unsigned char)src[e]) && src[e] != '(' && src[e] != ')' &&
               src[e] != ';')
            ++e;
        tok = src.substr(pos, e - pos);
        pos = e;
        return true;
    }
    bool is(const char *s) const { return tok == s; }
    std::string where() const { return file + ":" + std::to_string(tok_line); }
};

bool fail(const Lexer &L, const std::string &msg) {
    g_last_error = L.where() + ": " + msg + (L.tok.empty() ? " (end of file)" : " near '" + L.tok + "'");
    return false;
}

bool read_file(const char *path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

bool to_num(const std::string &s, double &v) {
    if (s.empty()) return false;
    char *end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return end && *end == '\0' && std::isfinite(v);
}

// skips to just past the next ';' (the current token included)
bool skip_statement(Lexer &L) {
    while (!L.is(";")) {
        if (!L.next()) return false;
    }
    return true;
}

// After an "END" token: true (past the pair) if the next token is `name`;
// a run of "END" tokens (a nested block closing right before) counts as one.
bool end_names(Lexer &L, const std::string &name, bool &ok) {
    ok = true;
    do {
        if (!L.next()) {
            ok = false;
            return false;
        }
    } while (L.is("END") && name != "END");
    return L.tok == name;
}

// skips to just past the pair "END <name>"
bool skip_to_end(Lexer &L, const std::string &name) {
    for (;;) {
        if (!L.next()) return false;
        if (L.is("END")) {
            bool ok;
            if (end_names(L, name, ok)) return true;
            if (!ok) return false;
        }
    }
}

// ---- LEF ---------------------------------------------------------------------
bool parse_lef(ap_design &d, const char *path) {
    Lexer L;
    L.file = path;
    if (!read_file(path, L.src)) {
        g_last_error = std::string(path) + ": cannot read";
        return false;
    }
    static const char *named_blocks[] = {"LAYER", "VIA", "VIARULE", "SITE", "NONDEFAULTRULE", "ARRAY"};
    static const char *keyword_blocks[] = {"UNITS", "SPACING", "PROPERTYDEFINITIONS", "NOISETABLE",
                                           "CORRECTIONTABLE", "IRDROP", "DIELECTRIC", "MAXVIASTACK"};
    while (L.next()) {
        if (L.is("MACRO")) {
            if (!L.next()) return fail(L, "MACRO without a name");
            const std::string name = L.tok;
            double sx = 0, sy = 0;
            bool have_size = false;
            for (;;) {
                if (!L.next()) return fail(L, "MACRO " + name + " not closed");
                if (L.is("END")) {
                    bool ok;
                    if (end_names(L, name, ok)) break;
                    if (!ok) return fail(L, "MACRO " + name + " not closed");
                    if (!L.is("SIZE")) continue;  // anything but SIZE needs no look
                }
                if (L.is("SIZE")) {
                    std::string a, by, b;
                    if (!L.next()) return fail(L, "SIZE");
                    a = L.tok;
                    if (!L.next()) return fail(L, "SIZE");
                    by = L.tok;
                    if (!L.next()) return fail(L, "SIZE");
                    b = L.tok;
                    if (by != "BY" || !to_num(a, sx) || !to_num(b, sy) || sx < 0 || sy < 0)
                        return fail(L, "malformed SIZE of MACRO " + name);
                    have_size = true;
                }
            }
            if (!have_size) return fail(L, "MACRO " + name + " has no SIZE");
            d.macros[name] = {sx, sy};  // a later definition replaces an earlier one
            continue;
        }
        bool done = false;
        for (const char *k : named_blocks)
            if (L.is(k)) {
                if (!L.next()) return fail(L, std::string(k) + " without a name");
                const std::string name = L.tok;
                // "LAYER name ;" inside other statements does not occur at top level
                if (!skip_to_end(L, name)) return fail(L, std::string(k) + " " + name + " not closed");
                done = true;
                break;
            }
        if (done) continue;
        for (const char *k : keyword_blocks)
            if (L.is(k)) {
                if (!skip_to_end(L, k)) return fail(L, std::string(k) + " not closed");
                done = true;
                break;
            }
        if (done) continue;
        if (L.is("BEGINEXT")) {
            while (L.next() && !L.is("ENDEXT")) {
            }
            continue;
        }
        if (L.is("END")) {
            if (!L.next()) break;
            if (L.is("LIBRARY")) break;
            continue;
        }
        if (!skip_statement(L)) return fail(L, "statement not closed by ';'");
    }
    return true;
}

// ---- DEF ---------------------------------------------------------------------
int status_of(const std::string &s) {
    if (s == "PLACED") return 1;
    if (s == "FIXED") return 2;
    if (s == "COVER") return 3;
    return 0;
}

bool read_point(Lexer &L, double &x, double &y) {
    if (!L.next() || !L.is("(")) return false;
    if (!L.next() || !to_num(L.tok, x)) return false;
    if (!L.next() || !to_num(L.tok, y)) return false;
    if (!L.next() || !L.is(")")) return false;
    return true;
}

bool parse_components(Lexer &L, ap_design &d) {
    for (;;) {
        if (!L.next()) return fail(L, "COMPONENTS not closed");
        if (L.is("END")) {
            if (!L.next() || !L.is("COMPONENTS")) return fail(L, "expected END COMPONENTS");
            return true;
        }
        if (!L.is("-")) return fail(L, "expected '-' starting a component");
        Component c{};
        if (!L.next()) return fail(L, "component name");
        c.name = L.tok;
        if (!L.next()) return fail(L, "component model");
        c.model = L.tok;
        c.orient = "N";
        if (!L.next()) return fail(L, "component " + c.name + " not closed");
        while (!L.is(";")) {
            if (L.is("+")) {
                if (!L.next()) return fail(L, "component attribute");
                const int st = status_of(L.tok);
                if (st) {
                    c.status = st;
                    if (!read_point(L, c.x, c.y)) return fail(L, "placement point of " + c.name);
                    if (!L.next()) return fail(L, "orientation of " + c.name);
                    c.orient = L.tok;
                } else if (L.is("UNPLACED")) {
                    c.status = 0;
                }
            }
            if (!L.next()) return fail(L, "component " + c.name + " not closed");
        }
        d.comps.push_back(std::move(c));
    }
}

bool parse_pins(Lexer &L, ap_design &d) {
    for (;;) {
        if (!L.next()) return fail(L, "PINS not closed");
        if (L.is("END")) {
            if (!L.next() || !L.is("PINS")) return fail(L, "expected END PINS");
            return true;
        }
        if (!L.is("-")) return fail(L, "expected '-' starting a pin");
        IoPin p{};
        if (!L.next()) return fail(L, "pin name");
        p.name = L.tok;
        p.orient = "N";
        if (!L.next()) return fail(L, "pin " + p.name + " not closed");
        while (!L.is(";")) {
            if (L.is("+")) {
                if (!L.next()) return fail(L, "pin attribute");
                const int st = status_of(L.tok);
                if (L.is("NET")) {
                    if (!L.next()) return fail(L, "NET of pin " + p.name);
                    p.net = L.tok;
                } else if (L.is("DIRECTION")) {
                    if (!L.next()) return fail(L, "DIRECTION of pin " + p.name);
                    p.direction = L.tok;
                } else if (L.is("USE")) {
                    if (!L.next()) return fail(L, "USE of pin " + p.name);
                    p.use = L.tok;
                } else if (L.is("LAYER")) {
                    if (!L.next()) return fail(L, "LAYER of pin " + p.name);
                    const std::string layer = L.tok;
                    // optional MASK / SPACING / DESIGNRULEWIDTH before the rectangle
                    double a, b, c2, e;
                    if (!L.next()) return fail(L, "LAYER of pin " + p.name);
                    while (!L.is("(")) {
                        if (L.is(";") || L.is("+")) return fail(L, "LAYER of pin " + p.name + " without a rectangle");
                        if (!L.next()) return fail(L, "LAYER of pin " + p.name);
                    }
                    // at '(': read two points
                    if (!L.next() || !to_num(L.tok, a)) return fail(L, "pin rectangle");
                    if (!L.next() || !to_num(L.tok, b)) return fail(L, "pin rectangle");
                    if (!L.next() || !L.is(")")) return fail(L, "pin rectangle");
                    if (!read_point(L, c2, e)) return fail(L, "pin rectangle");
                    if (!p.has_rect) {
                        p.has_rect = true;
                        p.layer = layer;
                        p.rect[0] = std::llround(a);
                        p.rect[1] = std::llround(b);
                        p.rect[2] = std::llround(c2);
                        p.rect[3] = std::llround(e);
                    }
                } else if (st) {
                    p.status = st;
                    if (!read_point(L, p.x, p.y)) return fail(L, "placement point of pin " + p.name);
                    if (!L.next()) return fail(L, "orientation of pin " + p.name);
                    p.orient = L.tok;
                }
            }
            if (!L.next()) return fail(L, "pin " + p.name + " not closed");
        }
        d.pins.push_back(std::move(p));
    }
}

bool parse_nets(Lexer &L, ap_design &d, const std::unordered_map<std::string, int> &comp_id,
                const std::unordered_map<std::string, int> &pin_id) {
    for (;;) {
        if (!L.next()) return fail(L, "NETS not closed");
        if (L.is("END")) {
            if (!L.next() || !L.is("NETS")) return fail(L, "expected END NETS");
            return true;
        }
        if (!L.is("-")) return fail(L, "expected '-' starting a net");
        Net n;
        if (!L.next()) return fail(L, "net name");
        n.name = L.tok;
        if (!L.next()) return fail(L, "net " + n.name + " not closed");
        bool attrs = false;  // past the first '+': routing and properties, skipped
        while (!L.is(";")) {
            if (L.is("+")) attrs = true;
            if (!attrs && L.is("(")) {
                if (!L.next()) return fail(L, "connection of net " + n.name);
                const std::string a = L.tok;
                if (!L.next()) return fail(L, "connection of net " + n.name);
                const std::string b = L.tok;
                if (!L.next()) return fail(L, "connection of net " + n.name);
                while (!L.is(")")) {  // "+ SYNTHESIZED" inside a connection
                    if (L.is(";")) return fail(L, "connection of net " + n.name + " not closed");
                    if (!L.next()) return fail(L, "connection of net " + n.name);
                }
                if (a == "PIN") {
                    auto it = pin_id.find(b);
                    if (it == pin_id.end()) return fail(L, "net " + n.name + " names unknown IO pin " + b);
                    n.conns.push_back({it->second, std::string()});
                } else if (a != "*") {
                    auto it = comp_id.find(a);
                    if (it == comp_id.end()) return fail(L, "net " + n.name + " names unknown component " + a);
                    n.conns.push_back({it->second, b});
                }
            }
            if (!L.next()) return fail(L, "net " + n.name + " not closed");
        }
        d.nets.push_back(std::move(n));
    }
}

bool parse_def(ap_design &d, const char *path) {
    Lexer L;
    L.file = path;
    if (!read_file(path, L.src)) {
        g_last_error = std::string(path) + ": cannot read";
        return false;
    }
    static const char *skip_sections[] = {"VIAS",        "SPECIALNETS", "BLOCKAGES",          "REGIONS",
                                          "GROUPS",      "FILLS",       "SCANCHAINS",         "NONDEFAULTRULES",
                                          "STYLES",      "SLOTS",       "PROPERTYDEFINITIONS", "PINPROPERTIES",
                                          "BEGINEXT"};
    std::unordered_map<std::string, int> comp_id, pin_id;
    while (L.next()) {
        if (L.is("DESIGN")) {
            if (!L.next()) return fail(L, "DESIGN without a name");
            d.design_name = L.tok;
            if (!L.next() || !skip_statement(L)) return fail(L, "DESIGN not closed");
        } else if (L.is("VERSION")) {
            if (!L.next()) return fail(L, "VERSION");
            d.def_version = L.tok;
            if (!L.next() || !skip_statement(L)) return fail(L, "VERSION not closed");
        } else if (L.is("UNITS")) {
            double u = 0;
            if (!L.next() || !L.is("DISTANCE") || !L.next() || !L.is("MICRONS") || !L.next() || !to_num(L.tok, u) ||
                !(u > 0))
                return fail(L, "expected UNITS DISTANCE MICRONS <n>");
            d.units = (int)std::llround(u);
            if (!L.next() || !skip_statement(L)) return fail(L, "UNITS not closed");
        } else if (L.is("DIEAREA")) {
            double xl = 1e300, yl = 1e300, xh = -1e300, yh = -1e300, px, py;
            int np = 0;
            for (;;) {
                const size_t save = L.pos;
                const int save_line = L.line;
                if (!L.next()) return fail(L, "DIEAREA not closed");
                if (L.is(";")) break;
                L.pos = save;
                L.line = save_line;
                if (!read_point(L, px, py)) return fail(L, "DIEAREA point");
                xl = std::min(xl, px);
                yl = std::min(yl, py);
                xh = std::max(xh, px);
                yh = std::max(yh, py);
                ++np;
            }
            if (np < 2 || !(xh > xl) || !(yh > yl)) return fail(L, "DIEAREA needs two corners of a non-empty box");
            d.die[0] = xl;
            d.die[1] = yl;
            d.die[2] = xh;
            d.die[3] = yh;
            d.has_die = true;
        } else if (L.is("COMPONENTS")) {
            if (!L.next() || !skip_statement(L)) return fail(L, "COMPONENTS count");
            if (!parse_components(L, d)) return false;
            for (size_t i = 0; i < d.comps.size(); ++i)
                if (!comp_id.emplace(d.comps[i].name, (int)i).second)
                    return fail(L, "component " + d.comps[i].name + " defined twice");
        } else if (L.is("PINS")) {
            if (!L.next() || !skip_statement(L)) return fail(L, "PINS count");
            if (!parse_pins(L, d)) return false;
        } else if (L.is("NETS")) {
            if (!L.next() || !skip_statement(L)) return fail(L, "NETS count");
            // IO pin nodes follow the components
            pin_id.clear();
            for (size_t i = 0; i < d.pins.size(); ++i)
                if (!pin_id.emplace(d.pins[i].name, (int)(d.comps.size() + i)).second)
                    return fail(L, "IO pin " + d.pins[i].name + " defined twice");
            if (!parse_nets(L, d, comp_id, pin_id)) return false;
        } else if (L.is("END")) {
            if (!L.next()) break;
            if (L.is("DESIGN")) break;
        } else {
            bool skipped = false;
            for (const char *k : skip_sections)
                if (L.is(k)) {
                    if (L.is("BEGINEXT")) {
                        while (L.next() && !L.is("ENDEXT")) {
                        }
                    } else if (!skip_to_end(L, k)) {
                        return fail(L, std::string(k) + " not closed");
                    }
                    skipped = true;
                    break;
                }
            if (!skipped && !skip_statement(L)) return fail(L, "statement not closed by ';'");
        }
    }
    if (!d.has_die) {
        g_last_error = std::string(path) + ": no DIEAREA";
        return false;
    }
    return true;
}

bool rotated(const std::string &o) { return o == "E" || o == "W" || o == "FE" || o == "FW"; }

bool build_netlist(ap_design &d) {
    const size_t nc = d.comps.size(), np = d.pins.size(), n = nc + np;
    d.w.assign(n, 0.f);
    d.h.assign(n, 0.f);
    d.x.assign(n, 0.f);
    d.y.assign(n, 0.f);
    d.fixed.assign(n, 0);
    const double scale = d.size_mode == AP_LEF_SIZE_DBU ? (double)d.units : 1.0;
    for (size_t i = 0; i < nc; ++i) {
        const Component &c = d.comps[i];
        auto it = d.macros.find(c.model);
        if (it == d.macros.end()) {
            g_last_error = "component " + c.name + ": model " + c.model + " not defined in the LEF files";
            return false;
        }
        double sw = it->second.first * scale, sh = it->second.second * scale;
        if (d.size_mode == AP_LEF_SIZE_DBU && rotated(c.orient)) std::swap(sw, sh);
        d.w[i] = (float)sw;
        d.h[i] = (float)sh;
        d.x[i] = (float)c.x;
        d.y[i] = (float)c.y;
        d.fixed[i] = c.status >= 2;
    }
    for (size_t k = 0; k < np; ++k) {
        d.x[nc + k] = (float)d.pins[k].x;
        d.y[nc + k] = (float)d.pins[k].y;
        d.fixed[nc + k] = 1;  // zero-area: pins only
    }
    d.net_ptr.assign(1, 0);
    d.pin_node.clear();
    for (const Net &e : d.nets) {
        for (const NetConn &q : e.conns) d.pin_node.push_back(q.node);
        d.net_ptr.push_back((int32_t)d.pin_node.size());
    }
    return true;
}

ap_design *read_design(const std::vector<std::string> &lefs, const std::string &def, int32_t size_mode) {
    g_last_error.clear();
    if (size_mode != AP_LEF_SIZE_DBU && size_mode != AP_LEF_SIZE_AS_READ) {
        g_last_error = "unknown LEF size mode";
        return nullptr;
    }
    ap_design *d = new ap_design();
    d->size_mode = size_mode;
    for (const std::string &l : lefs)
        if (!parse_lef(*d, l.c_str())) {
            delete d;
            return nullptr;
        }
    if (!parse_def(*d, def.c_str()) || !build_netlist(*d)) {
        delete d;
        return nullptr;
    }
    return d;
}

std::string fmt_coord(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%lld", (long long)std::llround(v));
    return b;
}

const char *status_name(int s) { return s == 2 ? "FIXED" : s == 3 ? "COVER" : "PLACED"; }

}  // namespace

extern "C" {

const char *ap_last_error(void) { return g_last_error.c_str(); }

__attribute__((visibility("hidden"))) void ap_internal_set_error(const char *msg) {
    g_last_error = msg ? msg : "";
}

int ap_design_read(const char *const *lef_paths, int32_t n_lef, const char *def_path, int32_t size_mode,
                   ap_design **out) {
    if (!out || !def_path || n_lef < 0 || (n_lef > 0 && !lef_paths)) return AP_ERR_INVALID_ARG;
    *out = nullptr;
    std::vector<std::string> lefs;
    for (int i = 0; i < n_lef; ++i) {
        if (!lef_paths[i]) return AP_ERR_INVALID_ARG;
        lefs.emplace_back(lef_paths[i]);
    }
    ap_design *d = read_design(lefs, def_path, size_mode);
    if (!d) return AP_ERR_BAD_NETLIST;
    *out = d;
    return AP_OK;
}

int ap_design_read_dir(const char *dir, int32_t size_mode, ap_design **out) {
    if (!dir || !out) return AP_ERR_INVALID_ARG;
    *out = nullptr;
    DIR *dp = opendir(dir);
    if (!dp) {
        g_last_error = std::string(dir) + ": cannot open the design directory";
        return AP_ERR_INVALID_ARG;
    }
    std::vector<std::string> lefs;
    bool have_def = false;
    while (dirent *e = readdir(dp)) {
        const std::string f = e->d_name;
        if (f.size() > 4 && f.compare(f.size() - 4, 4, ".lef") == 0) lefs.push_back(std::string(dir) + "/" + f);
        if (f == "floorplan.def") have_def = true;
    }
    closedir(dp);
    std::sort(lefs.begin(), lefs.end());  // a fixed order (readdir's is unspecified)
    if (lefs.empty() || !have_def) {
        g_last_error = std::string(dir) + ": needs *.lef files and floorplan.def";
        return AP_ERR_INVALID_ARG;
    }
    ap_design *d = read_design(lefs, std::string(dir) + "/floorplan.def", size_mode);
    if (!d) return AP_ERR_BAD_NETLIST;
    *out = d;
    return AP_OK;
}

int ap_design_get_info(ap_design *d, ap_design_info *info) {
    if (!d || !info) return AP_ERR_INVALID_ARG;
    info->num_nodes = (int32_t)d->w.size();
    info->num_nets = (int32_t)d->nets.size();
    info->num_pins = (int32_t)d->pin_node.size();
    info->num_components = (int32_t)d->comps.size();
    info->num_io_pins = (int32_t)d->pins.size();
    info->units_per_micron = d->units;
    info->die_xl = (float)d->die[0];
    info->die_yl = (float)d->die[1];
    info->die_xh = (float)d->die[2];
    info->die_yh = (float)d->die[3];
    return AP_OK;
}

int ap_design_netlist(ap_design *d, ap_netlist *nl) {
    if (!d || !nl) return AP_ERR_INVALID_ARG;
    nl->num_nodes = (int32_t)d->w.size();
    nl->num_nets = (int32_t)d->nets.size();
    nl->num_pins = (int32_t)d->pin_node.size();
    nl->net_ptr = d->net_ptr.data();
    nl->pin_node = d->pin_node.data();
    nl->node_w = d->w.data();
    nl->node_h = d->h.data();
    nl->node_x = d->x.data();
    nl->node_y = d->y.data();
    nl->node_fixed = d->fixed.data();
    nl->die_xl = (float)d->die[0];
    nl->die_yl = (float)d->die[1];
    nl->die_xh = (float)d->die[2];
    nl->die_yh = (float)d->die[3];
    return AP_OK;
}

const char *ap_design_node_name(ap_design *d, int32_t i) {
    if (!d || i < 0) return nullptr;
    const size_t k = (size_t)i;
    if (k < d->comps.size()) return d->comps[k].name.c_str();
    if (k < d->comps.size() + d->pins.size()) return d->pins[k - d->comps.size()].name.c_str();
    return nullptr;
}

const char *ap_design_name(ap_design *d) { return d ? d->design_name.c_str() : nullptr; }

int ap_design_write_def(ap_design *d, const float *x, const float *y, const char *path) {
    if (!d || !x || !y || !path) return AP_ERR_INVALID_ARG;
    const size_t nc = d->comps.size(), np = d->pins.size();
    for (size_t i = 0; i < nc; ++i)
        if (!std::isfinite(x[i]) || !std::isfinite(y[i])) return AP_ERR_NONFINITE;
    std::ofstream out(path);
    if (!out) {
        g_last_error = std::string(path) + ": cannot write";
        return AP_ERR_INVALID_ARG;
    }
    out << "# Design after global placement\n# Written by the GB300 ePlace library\n";
    out << "VERSION 5.8 ;\nDIVIDERCHAR \"/\" ;\nBUSBITCHARS \"[]\" ;\n";
    out << "DESIGN " << (d->design_name.empty() ? "design" : d->design_name) << " ;\n";
    out << "UNITS DISTANCE MICRONS " << d->units << " ;\n\n";
    out << "DIEAREA ( " << fmt_coord(d->die[0]) << " " << fmt_coord(d->die[1]) << " ) ( " << fmt_coord(d->die[2])
        << " " << fmt_coord(d->die[3]) << " ) ;\n\n";
    out << "COMPONENTS " << nc << " ;\n";
    for (size_t i = 0; i < nc; ++i) {
        const Component &c = d->comps[i];
        // fixed components keep their place; the rest at the placed position
        const double px = c.status >= 2 ? c.x : (double)x[i], py = c.status >= 2 ? c.y : (double)y[i];
        out << "    - " << c.name << " " << c.model << "\n      + " << status_name(c.status) << " ( " << fmt_coord(px)
            << " " << fmt_coord(py) << " ) " << c.orient << " ;\n";
    }
    out << "END COMPONENTS\n\n";
    out << "PINS " << np << " ;\n";
    for (size_t k = 0; k < np; ++k) {
        const IoPin &p = d->pins[k];
        out << "    - " << p.name << " + NET " << (p.net.empty() ? p.name : p.net);
        if (!p.direction.empty()) out << "\n      + DIRECTION " << p.direction;
        if (!p.use.empty()) out << "\n      + USE " << p.use;
        if (p.has_rect)
            out << "\n      + LAYER " << p.layer << " ( " << p.rect[0] << " " << p.rect[1] << " ) ( " << p.rect[2]
                << " " << p.rect[3] << " )";
        if (p.status) out << "\n      + " << status_name(p.status) << " ( " << fmt_coord(p.x) << " " << fmt_coord(p.y)
                          << " ) " << p.orient;
        out << " ;\n";
    }
    out << "END PINS\n\n";
    out << "NETS " << d->nets.size() << " ;\n";
    for (const Net &e : d->nets) {
        out << "    - " << e.name;
        int count = 0;
        for (const NetConn &q : e.conns) {
            if ((size_t)q.node >= nc)
                out << " ( PIN " << d->pins[(size_t)q.node - nc].name << " )";
            else
                out << " ( " << d->comps[(size_t)q.node].name << " " << q.pin << " )";
            if (++count == 4 && &q != &e.conns.back()) {  // four connections a line
                out << "\n     ";
                count = 0;
            }
        }
        out << " ;\n";
    }
    out << "END NETS\n\nEND DESIGN\n";
    out.close();
    return out ? AP_OK : AP_ERR_INVALID_ARG;
}

int ap_design_destroy(ap_design *d) {
    if (!d) return AP_ERR_INVALID_ARG;
    delete d;
    return AP_OK;
}

}  // extern "C"
