// Run configuration from JSON, the placer's counterpart of the reference
// host's config file (vck5000/host/config_aieplace.json, read by
// Placer::Placer, AIEplace.cpp:87-109).  Host code.
//
// The keys sit under "params" as in the reference file (or at the top
// level).  Reference keys and how they map:
//   use_aie              accepted; this placer has no AIE path (ignored)
//   input_filepath       design directory: *.lef + floorplan.def
//   output_filepath      directory of the placed DEF (<design>.def)
//   wirelength_method    "HPWL" or "WA": the wirelength the run reports
//   bins_per_row         bins_x = bins_y
//   gamma                gamma_base_bins (the WA smoothing in bins; the loop
//                        scales it with the overflow, RePlAce)
//   max_iterations       max_iterations
//   init_learning_rate   accepted, ignored: the Nesterov loop predicts its
//                        step lengths (Lipschitz), it has no fixed rate
//   init_global_lambda   init_density_weight when > 0 (0 keeps the default;
//                        the reference's 0 would leave the density term off)
// Keys of this placer: every ap_params field by name (target_density,
// gamma_base_bins, field_solver "fp32"|"bf16x3", init_density_weight,
// ref_delta_hpwl, lambda_mu_max, lambda_mu_min, init_step_coef,
// target_overflow, check_interval, use_graph, max_backtracks, restart_mode),
// and log_path, lef_size_mode ("dbu"|"as_read"), seed, init_sigma,
// filler_cells.  Unknown keys are errors.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

#include "../../include/aieplace.h"

// the thread's last error message (lefdef.cpp), read through ap_last_error
extern "C" __attribute__((visibility("hidden"))) void ap_internal_set_error(const char *msg);

namespace {

// A JSON value: only what a flat config needs (objects, strings, numbers,
// booleans, null; arrays are parsed and rejected where a key needs a scalar).
struct JVal {
    enum Kind { NUL, BOOL, NUM, STR, OBJ, ARR } kind = NUL;
    double num = 0;
    bool b = false;
    std::string str;
    std::map<std::string, JVal> obj;
    int line = 0;
};

struct JParser {
    const std::string &s;
    size_t p = 0;
    int line = 1;
    std::string err;

    explicit JParser(const std::string &src) : s(src) {}

    void ws() {
        while (p < s.size() && (s[p] == ' ' || s[p] == '\t' || s[p] == '\n' || s[p] == '\r')) {
            if (s[p] == '\n') ++line;
            ++p;
        }
    }
    bool fail(const std::string &m) {
        if (err.empty()) err = "line " + std::to_string(line) + ": " + m;
        return false;
    }
    bool str(std::string &out) {
        if (p >= s.size() || s[p] != '"') return fail("expected a string");
        ++p;
        out.clear();
        while (p < s.size() && s[p] != '"') {
            char c = s[p++];
            if (c == '\\' && p < s.size()) {
                const char e = s[p++];
                c = e == 'n' ? '\n' : e == 't' ? '\t' : e;
            }
            out.push_back(c);
        }
        if (p >= s.size()) return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(JVal &v) {
        ws();
        if (p >= s.size()) return fail("unexpected end of input");
        v.line = line;
        const char c = s[p];
        if (c == '{') {
            v.kind = JVal::OBJ;
            ++p;
            ws();
            if (p < s.size() && s[p] == '}') {
                ++p;
                return true;
            }
            for (;;) {
                ws();
                std::string k;
                if (!str(k)) return false;
                ws();
                if (p >= s.size() || s[p] != ':') return fail("expected ':'");
                ++p;
                JVal child;
                if (!value(child)) return false;
                v.obj[k] = child;
                ws();
                if (p < s.size() && s[p] == ',') {
                    ++p;
                    continue;
                }
                if (p < s.size() && s[p] == '}') {
                    ++p;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = JVal::ARR;
            ++p;
            int depth = 1;
            while (p < s.size() && depth) {  // contents are not needed
                if (s[p] == '[') ++depth;
                if (s[p] == ']') --depth;
                if (s[p] == '\n') ++line;
                ++p;
            }
            return depth == 0 || fail("unterminated array");
        }
        if (c == '"') {
            v.kind = JVal::STR;
            return str(v.str);
        }
        if (s.compare(p, 4, "true") == 0) {
            v.kind = JVal::BOOL;
            v.b = true;
            p += 4;
            return true;
        }
        if (s.compare(p, 5, "false") == 0) {
            v.kind = JVal::BOOL;
            p += 5;
            return true;
        }
        if (s.compare(p, 4, "null") == 0) {
            p += 4;
            return true;
        }
        const char *start = s.c_str() + p;
        char *end = nullptr;
        v.num = std::strtod(start, &end);
        if (end == start) return fail("unexpected character");
        v.kind = JVal::NUM;
        p += (size_t)(end - start);
        return true;
    }
};

bool num(const JVal &v, double &out) {
    if (v.kind == JVal::NUM) {
        out = v.num;
        return true;
    }
    if (v.kind == JVal::BOOL) {
        out = v.b ? 1.0 : 0.0;
        return true;
    }
    return false;
}

bool copy_str(const JVal &v, char *dst, size_t cap) {
    if (v.kind != JVal::STR || v.str.size() + 1 > cap) return false;
    std::memcpy(dst, v.str.c_str(), v.str.size() + 1);
    return true;
}

}  // namespace

extern "C" int ap_run_config_default(ap_params *params, ap_run_config *run) {
    if (!params || !run) return AP_ERR_INVALID_ARG;
    ap_params_default(params);
    std::memset(run, 0, sizeof(*run));
    std::strcpy(run->output_dir, ".");
    run->size_mode = AP_LEF_SIZE_DBU;
    run->wirelength_method = 0;
    run->init_sigma = 0.f;  // one bin width
    run->seed = 1;
    run->filler_cells = 0;
    run->use_aie = 0;
    return AP_OK;
}

extern "C" int ap_run_config_read(const char *path, ap_params *params, ap_run_config *run) {
    if (!path || !params || !run) return AP_ERR_INVALID_ARG;
    std::ifstream f(path);
    if (!f) {
        ap_internal_set_error((std::string(path) + ": cannot read").c_str());
        return AP_ERR_INVALID_ARG;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string src = ss.str();
    JParser jp(src);
    JVal root;
    auto err = [&](const std::string &m) {
        ap_internal_set_error((std::string(path) + ": " + m).c_str());
        return AP_ERR_INVALID_ARG;
    };
    if (!jp.value(root)) return err(jp.err);
    jp.ws();
    if (jp.p != src.size()) return err("trailing characters after the JSON value");
    if (root.kind != JVal::OBJ) return err("the config is not a JSON object");
    ap_run_config_default(params, run);
    const std::map<std::string, JVal> *keys = &root.obj;
    auto it = root.obj.find("params");
    if (it != root.obj.end()) {
        if (it->second.kind != JVal::OBJ) return err("\"params\" is not an object");
        keys = &it->second.obj;
    }
    for (const auto &kv : *keys) {
        const std::string &k = kv.first;
        const JVal &v = kv.second;
        const std::string at = "key \"" + k + "\" (line " + std::to_string(v.line) + ")";
        double d = 0;
        // reference keys
        if (k == "use_aie") {
            if (!num(v, d)) return err(at + ": expected a boolean");
            run->use_aie = d != 0;
        } else if (k == "input_filepath") {
            if (!copy_str(v, run->input_dir, sizeof run->input_dir)) return err(at + ": expected a path");
        } else if (k == "output_filepath") {
            if (!copy_str(v, run->output_dir, sizeof run->output_dir)) return err(at + ": expected a path");
        } else if (k == "wirelength_method") {
            if (v.kind != JVal::STR || (v.str != "HPWL" && v.str != "WA")) return err(at + ": expected \"HPWL\" or \"WA\"");
            run->wirelength_method = v.str == "WA";
        } else if (k == "bins_per_row") {
            if (!num(v, d) || d != std::floor(d)) return err(at + ": expected an integer");
            params->bins_x = params->bins_y = (int32_t)d;
        } else if (k == "gamma" || k == "gamma_base_bins") {
            if (!num(v, d) || !(d > 0)) return err(at + ": expected a positive number");
            params->gamma_base_bins = (float)d;
        } else if (k == "max_iterations") {
            if (!num(v, d) || d != std::floor(d) || d < 0) return err(at + ": expected a non-negative integer");
            params->max_iterations = (int32_t)d;
        } else if (k == "init_learning_rate") {
            if (!num(v, d)) return err(at + ": expected a number");
            run->ignored_learning_rate = (float)d;
        } else if (k == "init_global_lambda") {
            if (!num(v, d) || d < 0) return err(at + ": expected a non-negative number");
            if (d > 0) params->init_density_weight = (float)d;
        }
        // this placer's keys
        else if (k == "target_density") {
            if (!num(v, d) || !(d > 0) || d > 1) return err(at + ": expected a number in (0, 1]");
            params->target_density = (float)d;
        } else if (k == "field_solver") {
            if (v.kind != JVal::STR || (v.str != "fp32" && v.str != "bf16x3")) return err(at + ": expected \"fp32\" or \"bf16x3\"");
            params->field_solver = v.str == "bf16x3" ? AP_FIELD_BF16X3 : AP_FIELD_FP32;
        } else if (k == "init_density_weight" || k == "ref_delta_hpwl" || k == "lambda_mu_max" || k == "lambda_mu_min" ||
                   k == "init_step_coef" || k == "target_overflow") {
            if (!num(v, d)) return err(at + ": expected a number");
            float *dst = k == "init_density_weight" ? &params->init_density_weight
                         : k == "ref_delta_hpwl"    ? &params->ref_delta_hpwl
                         : k == "lambda_mu_max"     ? &params->lambda_mu_max
                         : k == "lambda_mu_min"     ? &params->lambda_mu_min
                         : k == "init_step_coef"    ? &params->init_step_coef
                                                    : &params->target_overflow;
            *dst = (float)d;
        } else if (k == "check_interval" || k == "use_graph" || k == "max_backtracks" || k == "restart_mode") {
            if (!num(v, d) || d != std::floor(d) || d < 0) return err(at + ": expected a non-negative integer");
            int32_t *dst = k == "check_interval"   ? &params->check_interval
                           : k == "use_graph"      ? &params->use_graph
                           : k == "max_backtracks" ? &params->max_backtracks
                                                   : &params->restart_mode;
            *dst = (int32_t)d;
        } else if (k == "log_path") {
            if (!copy_str(v, run->log_path, sizeof run->log_path)) return err(at + ": expected a path");
        } else if (k == "lef_size_mode") {
            if (v.kind != JVal::STR || (v.str != "dbu" && v.str != "as_read")) return err(at + ": expected \"dbu\" or \"as_read\"");
            run->size_mode = v.str == "as_read" ? AP_LEF_SIZE_AS_READ : AP_LEF_SIZE_DBU;
        } else if (k == "seed") {
            if (!num(v, d) || d < 0 || d != std::floor(d)) return err(at + ": expected a non-negative integer");
            run->seed = (uint64_t)d;
        } else if (k == "init_sigma") {
            if (!num(v, d) || d < 0) return err(at + ": expected a non-negative number");
            run->init_sigma = (float)d;
        } else if (k == "filler_cells") {
            if (!num(v, d)) return err(at + ": expected a boolean");
            run->filler_cells = d != 0;
        } else {
            return err("unknown " + at);
        }
    }
    return AP_OK;
}
