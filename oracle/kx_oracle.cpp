// kx_oracle.cpp — THE ORACLE. Test infrastructure only.
//
// A CPU restatement of the pricing path of LePhilippeDucTai/kontracts (crate
// `kontract` 0.2.3, Rust). It is used by tests/, by the smoke check and by the
// CPU-baseline leg of bench.py as the checker and the timed CPU reference.
// The product (kontracts_gb300/) never links, imports or calls it.
//
// It keeps the reference's structure on purpose: parse the serde JSON into an
// AST, compile it to a Plan and a time grid, MATERIALISE every path on the
// grid, then reduce each path to cash flows by the recursive tree walk of
// pricer.rs and summarise with the two-pass formulas. Paths are processed in
// chunks so memory stays bounded; per-path results do not depend on chunking.
//
// Normals: the reference draws them from ChaCha8Rng::seed_from_u64(mix(seed, i))
// + rand_distr::StandardNormal (simulator.rs:233-241). Those come from the
// third-party crates rand_chacha 0.3 / rand_distr 0.4, which are not in the
// reference tree and are not pinned (no Cargo.lock), so bitwise stream parity
// with the reference is unpinned. The oracle instead takes its normals from
// (a) the same Philox4x32-10 + Box-Muller stream the GPU engine uses, or
// (b) host "shared draws" given by the caller. Parity with the reference is
// anchored on its own tests (sigma = 0 exact cases, closed forms, CRR trees).
//
// Compile with -ffp-contract=off so that x86 and Arm builds round like the
// reference (Rust never contracts a*b+c into an FMA).

#include "../include/kontract_gpu.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Errors (KontractError, src/error.rs:6-28)
// ---------------------------------------------------------------------------
struct KxError {
    int code;
    std::string msg;
};
thread_local std::string g_last_error;

[[noreturn]] void fail(int code, const std::string &msg) { throw KxError{code, msg}; }

// ---------------------------------------------------------------------------
// Minimal JSON DOM
// ---------------------------------------------------------------------------
struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
};

struct JParser {
    const char *p;
    const char *end;
    void ws() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    }
    [[noreturn]] void bad(const char *what) { fail(KX_SERDE, std::string("json: ") + what); }
    JVal parse() {
        ws();
        if (p >= end) bad("unexpected end");
        JVal v;
        char c = *p;
        if (c == '{') {
            v.kind = JVal::Obj;
            ++p;
            ws();
            if (p < end && *p == '}') { ++p; return v; }
            while (true) {
                ws();
                if (p >= end || *p != '"') bad("expected key");
                std::string k = parse_string();
                ws();
                if (p >= end || *p != ':') bad("expected ':'");
                ++p;
                v.obj.emplace_back(k, parse());
                ws();
                if (p < end && *p == ',') { ++p; continue; }
                if (p < end && *p == '}') { ++p; break; }
                bad("expected ',' or '}'");
            }
        } else if (c == '[') {
            v.kind = JVal::Arr;
            ++p;
            ws();
            if (p < end && *p == ']') { ++p; return v; }
            while (true) {
                v.arr.push_back(parse());
                ws();
                if (p < end && *p == ',') { ++p; continue; }
                if (p < end && *p == ']') { ++p; break; }
                bad("expected ',' or ']'");
            }
        } else if (c == '"') {
            v.kind = JVal::Str;
            v.str = parse_string();
        } else if (c == 't' && end - p >= 4 && !strncmp(p, "true", 4)) {
            v.kind = JVal::Bool; v.b = true; p += 4;
        } else if (c == 'f' && end - p >= 5 && !strncmp(p, "false", 5)) {
            v.kind = JVal::Bool; v.b = false; p += 5;
        } else if (c == 'n' && end - p >= 4 && !strncmp(p, "null", 4)) {
            v.kind = JVal::Null; p += 4;
        } else if (c == '-' || (c >= '0' && c <= '9')) {
            const char *s = p;
            if (*p == '-') ++p;
            while (p < end && ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' || *p == 'E' ||
                               *p == '+' || *p == '-'))
                ++p;
            std::string tok(s, p);
            char *ep = nullptr;
            v.num = strtod(tok.c_str(), &ep);
            if (!ep || *ep) bad("bad number");
            v.kind = JVal::Num;
        } else {
            bad("unexpected character");
        }
        return v;
    }
    std::string parse_string() {
        ++p;  // opening quote
        std::string out;
        while (p < end && *p != '"') {
            if (*p == '\\') {
                ++p;
                if (p >= end) bad("bad escape");
                char e = *p++;
                switch (e) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    if (end - p < 4) bad("bad \\u");
                    unsigned cp = (unsigned)strtoul(std::string(p, p + 4).c_str(), nullptr, 16);
                    p += 4;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                    else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                    break;
                }
                default: bad("bad escape");
                }
            } else {
                out += *p++;
            }
        }
        if (p >= end) bad("unterminated string");
        ++p;
        return out;
    }
};

// ---------------------------------------------------------------------------
// AST (src/ast.rs:34-206)
// ---------------------------------------------------------------------------
struct Obs;
struct Cond;
struct Con;
using ObsP = std::unique_ptr<Obs>;
using CondP = std::unique_ptr<Cond>;
using ConP = std::unique_ptr<Con>;

enum ObsK { O_CONST, O_SPOT, O_NEG, O_ADD, O_SUB, O_MUL, O_DIV, O_MAX, O_MIN, O_AVG, O_RMAX, O_RMIN };
struct Obs {
    ObsK k;
    double c = 0;
    std::string name;
    ObsP a, b;
    bool has_from = false, has_to = false;
    double from = 0, to = 0;
};
enum CondK { C_BOOL, C_AT, C_GE, C_GT, C_LE, C_LT, C_AND, C_OR, C_NOT };
struct Cond {
    CondK k;
    bool b = false;
    double t = 0;
    ObsP l, r;
    CondP x, y;
};
enum ConK { K_ZERO, K_ONE, K_GIVE, K_AND, K_OR, K_SCALE, K_WHEN, K_ANYTIME, K_UNTIL };
struct Con {
    ConK k;
    std::string ccy;
    ObsP obs;
    CondP cond;
    ConP a, b;
};

// serde externally tagged enums: "Unit" or {"Variant": payload}.
const JVal &variant(const JVal &v, std::string &tag) {
    static const JVal null_v;
    if (v.kind == JVal::Str) { tag = v.str; return null_v; }
    if (v.kind != JVal::Obj || v.obj.size() != 1) fail(KX_SERDE, "expected a single-key enum object");
    tag = v.obj[0].first;
    return v.obj[0].second;
}
double num(const JVal &v) {
    if (v.kind != JVal::Num) fail(KX_SERDE, "expected a number");
    return v.num;
}
const JVal &pair_at(const JVal &v, int i) {
    if (v.kind != JVal::Arr || v.arr.size() != 2) fail(KX_SERDE, "expected a 2-element array");
    return v.arr[i];
}

ObsP to_obs(const JVal &v) {
    std::string tag;
    const JVal &pl = variant(v, tag);
    auto o = std::make_unique<Obs>();
    auto bin = [&](ObsK k) { o->k = k; o->a = to_obs(pair_at(pl, 0)); o->b = to_obs(pair_at(pl, 1)); };
    if (tag == "Const") { o->k = O_CONST; o->c = num(pl); }
    else if (tag == "Spot") { if (pl.kind != JVal::Str) fail(KX_SERDE, "Spot expects a string"); o->k = O_SPOT; o->name = pl.str; }
    else if (tag == "Neg") { o->k = O_NEG; o->a = to_obs(pl); }
    else if (tag == "Add") bin(O_ADD);
    else if (tag == "Sub") bin(O_SUB);
    else if (tag == "Mul") bin(O_MUL);
    else if (tag == "Div") bin(O_DIV);
    else if (tag == "Max") bin(O_MAX);
    else if (tag == "Min") bin(O_MIN);
    else if (tag == "RunningMax") { o->k = O_RMAX; o->a = to_obs(pl); }
    else if (tag == "RunningMin") { o->k = O_RMIN; o->a = to_obs(pl); }
    else if (tag == "Average") {
        o->k = O_AVG;
        const JVal *obs = nullptr, *fr = nullptr, *to = nullptr;
        if (pl.kind == JVal::Obj) {
            for (auto &kv : pl.obj) {
                if (kv.first == "obs") obs = &kv.second;
                else if (kv.first == "from_year") fr = &kv.second;
                else if (kv.first == "to_year") to = &kv.second;
                else fail(KX_SERDE, "unknown field in Average: " + kv.first);
            }
        } else if (pl.kind == JVal::Arr && pl.arr.size() == 3) {
            obs = &pl.arr[0]; fr = &pl.arr[1]; to = &pl.arr[2];
        } else fail(KX_SERDE, "bad Average payload");
        if (!obs) fail(KX_SERDE, "missing field `obs`");
        o->a = to_obs(*obs);
        if (fr && fr->kind != JVal::Null) { o->has_from = true; o->from = num(*fr); }
        if (to && to->kind != JVal::Null) { o->has_to = true; o->to = num(*to); }
    } else fail(KX_SERDE, "unknown variant `" + tag + "` of Observable");
    return o;
}

CondP to_cond(const JVal &v) {
    std::string tag;
    const JVal &pl = variant(v, tag);
    auto c = std::make_unique<Cond>();
    auto cmp = [&](CondK k) { c->k = k; c->l = to_obs(pair_at(pl, 0)); c->r = to_obs(pair_at(pl, 1)); };
    if (tag == "Bool") { if (pl.kind != JVal::Bool) fail(KX_SERDE, "Bool expects a boolean"); c->k = C_BOOL; c->b = pl.b; }
    else if (tag == "At") { c->k = C_AT; c->t = num(pl); }
    else if (tag == "Ge") cmp(C_GE);
    else if (tag == "Gt") cmp(C_GT);
    else if (tag == "Le") cmp(C_LE);
    else if (tag == "Lt") cmp(C_LT);
    else if (tag == "And") { c->k = C_AND; c->x = to_cond(pair_at(pl, 0)); c->y = to_cond(pair_at(pl, 1)); }
    else if (tag == "Or") { c->k = C_OR; c->x = to_cond(pair_at(pl, 0)); c->y = to_cond(pair_at(pl, 1)); }
    else if (tag == "Not") { c->k = C_NOT; c->x = to_cond(pl); }
    else fail(KX_SERDE, "unknown variant `" + tag + "` of Condition");
    return c;
}

ConP to_con(const JVal &v) {
    std::string tag;
    const JVal &pl = variant(v, tag);
    auto c = std::make_unique<Con>();
    auto two = [&](ConK k) { c->k = k; c->a = to_con(pair_at(pl, 0)); c->b = to_con(pair_at(pl, 1)); };
    auto cond_con = [&](ConK k) { c->k = k; c->cond = to_cond(pair_at(pl, 0)); c->a = to_con(pair_at(pl, 1)); };
    if (tag == "Zero") { if (v.kind != JVal::Str && pl.kind != JVal::Null) fail(KX_SERDE, "Zero takes no payload"); c->k = K_ZERO; }
    else if (tag == "One") { if (pl.kind != JVal::Str) fail(KX_SERDE, "One expects a currency string"); c->k = K_ONE; c->ccy = pl.str; }
    else if (tag == "Give") { c->k = K_GIVE; c->a = to_con(pl); }
    else if (tag == "And") two(K_AND);
    else if (tag == "Or") two(K_OR);
    else if (tag == "Scale") { c->k = K_SCALE; c->obs = to_obs(pair_at(pl, 0)); c->a = to_con(pair_at(pl, 1)); }
    else if (tag == "When") cond_con(K_WHEN);
    else if (tag == "Anytime") cond_con(K_ANYTIME);
    else if (tag == "Until") cond_con(K_UNTIL);
    else fail(KX_SERDE, "unknown variant `" + tag + "` of Contract");
    if (v.kind == JVal::Str && tag != "Zero") fail(KX_SERDE, "variant `" + tag + "` needs a payload");
    return c;
}

ConP parse_contract(const char *json) {
    if (!json) fail(KX_INVALID_ARGUMENT, "null contract json");
    JParser jp{json, json + strlen(json)};
    JVal v = jp.parse();
    jp.ws();
    if (jp.p != jp.end) fail(KX_SERDE, "json: trailing characters");
    return to_con(v);
}

// ---------------------------------------------------------------------------
// Compiler (src/compiler.rs:25-189)
// ---------------------------------------------------------------------------
struct Plan {
    std::vector<std::string> assets;
    std::vector<double> fixed_dates;
    double horizon = 0;
    bool needs_fine = false;
};

// compiler.rs:185-189 — sort, then drop values within 1e-12 of the last kept one.
std::vector<double> sort_dedup(std::vector<double> v) {
    std::sort(v.begin(), v.end());
    std::vector<double> out;
    for (double x : v)
        if (out.empty() || !(std::fabs(x - out.back()) < 1e-12)) out.push_back(x);
    return out;
}

struct Acc {
    std::set<std::string> assets;
    std::vector<double> dates;
    bool fine = false;
};

void walk_obs(const Obs &o, Acc &acc) {  // compiler.rs:123-146
    switch (o.k) {
    case O_CONST: break;
    case O_SPOT: acc.assets.insert(o.name); break;
    case O_NEG: walk_obs(*o.a, acc); break;
    case O_AVG: case O_RMAX: case O_RMIN: acc.fine = true; walk_obs(*o.a, acc); break;
    default: walk_obs(*o.a, acc); walk_obs(*o.b, acc);
    }
}
bool price_dependent(const Cond &c) {  // compiler.rs:173-182
    switch (c.k) {
    case C_BOOL: case C_AT: return false;
    case C_GE: case C_GT: case C_LE: case C_LT: return true;
    case C_AND: case C_OR: return price_dependent(*c.x) || price_dependent(*c.y);
    case C_NOT: return price_dependent(*c.x);
    }
    return false;
}
void walk_cond(const Cond &c, Acc &acc) {  // compiler.rs:148-169
    switch (c.k) {
    case C_BOOL: break;
    case C_AT:
        if (!std::isfinite(c.t) || c.t < 0.0) {
            char buf[96];
            snprintf(buf, sizeof buf, "invalid acquisition date: %g", c.t);
            fail(KX_MALFORMED_CONTRACT, buf);
        }
        acc.dates.push_back(c.t);
        break;
    case C_GE: case C_GT: case C_LE: case C_LT: walk_obs(*c.l, acc); walk_obs(*c.r, acc); break;
    case C_AND: case C_OR: walk_cond(*c.x, acc); walk_cond(*c.y, acc); break;
    case C_NOT: walk_cond(*c.x, acc); break;
    }
}
void walk_con(const Con &c, Acc &acc) {  // compiler.rs:95-121
    switch (c.k) {
    case K_ZERO: case K_ONE: break;
    case K_GIVE: walk_con(*c.a, acc); break;
    case K_AND: case K_OR: walk_con(*c.a, acc); walk_con(*c.b, acc); break;
    case K_SCALE: walk_obs(*c.obs, acc); walk_con(*c.a, acc); break;
    case K_WHEN: case K_ANYTIME: case K_UNTIL:
        walk_cond(*c.cond, acc);
        if (price_dependent(*c.cond)) acc.fine = true;
        walk_con(*c.a, acc);
        break;
    }
}
Plan compile(const Con &c) {  // compiler.rs:69-86
    Acc acc;
    walk_con(c, acc);
    Plan p;
    p.horizon = 0.0;
    for (double d : acc.dates) if (d > p.horizon) p.horizon = d;
    p.assets.assign(acc.assets.begin(), acc.assets.end());
    p.fixed_dates = sort_dedup(acc.dates);
    p.needs_fine = acc.fine;
    return p;
}
// compiler.rs:54-65
std::vector<double> time_grid_forced(const Plan &p, uint32_t spy, bool force) {
    std::vector<double> pts{0.0};
    pts.insert(pts.end(), p.fixed_dates.begin(), p.fixed_dates.end());
    pts.push_back(p.horizon);
    if ((p.needs_fine || force) && p.horizon > 0.0 && spy > 0) {
        size_t n = (size_t)std::ceil(p.horizon * (double)spy);
        for (size_t k = 1; k <= n; ++k) pts.push_back(p.horizon * (double)k / (double)n);
    }
    return sort_dedup(pts);
}

// ---------------------------------------------------------------------------
// Normal sources: Philox4x32-10 (Salmon et al., SC'11) + Box-Muller, or
// caller-provided shared draws.
// ---------------------------------------------------------------------------
inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[1] = (uint32_t)p1;
        c[3] = (uint32_t)p0;
        c[0] = n0;
        c[2] = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Draw d of path p: Philox block d/4 with counter (d/4, p_lo, p_hi, stream),
// key (seed_lo, seed_hi); words (w0,w1) give normals 0,1 and (w2,w3) give 2,3
// by Box-Muller: r = sqrt(-2 ln u1), th = 2 pi u2, (r cos th, r sin th),
// u = (w + 0.5) * 2^-32.
struct NormalSource {
    uint64_t seed = 0;
    uint32_t stream = 0;
    const double *shared = nullptr;  // path-major
    uint64_t shared_paths = 0, shared_dpp = 0;

    void fill(uint64_t path, size_t n_draws, double *out) const {
        if (shared) {
            if (path >= shared_paths || n_draws > shared_dpp)
                fail(KX_INVALID_ARGUMENT, "shared draws too small for this simulation");
            memcpy(out, shared + path * shared_dpp, n_draws * sizeof(double));
            return;
        }
        for (size_t blk = 0; blk * 4 < n_draws; ++blk) {
            uint32_t c[4] = {(uint32_t)blk, (uint32_t)path, (uint32_t)(path >> 32), stream};
            philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
            for (int h = 0; h < 2; ++h) {
                double u1 = ((double)c[2 * h] + 0.5) * 0x1p-32;
                double u2 = ((double)c[2 * h + 1] + 0.5) * 0x1p-32;
                double r = std::sqrt(-2.0 * std::log(u1));
                double th = 2.0 * M_PI * u2;
                size_t d0 = blk * 4 + 2 * h;
                if (d0 < n_draws) out[d0] = r * std::cos(th);
                if (d0 + 1 < n_draws) out[d0 + 1] = r * std::sin(th);
            }
        }
    }
};

// ---------------------------------------------------------------------------
// Models and simulation (src/simulator.rs)
// ---------------------------------------------------------------------------
struct Model {
    int kind = KX_MODEL_GBM;
    int scheme = KX_HESTON_REFERENCE_FLOOR;
    double s0 = 100, mu = 0, sigma = 0.2;
    double v0 = 0.04, kappa = 1, theta = 0.04, sigma_v = 0, rho = 0, r = 0;
    std::string asset = "ASSET";
    bool requires_fine() const { return kind == KX_MODEL_HESTON; }  // simulator.rs:546
    size_t draws_per_step() const { return kind == KX_MODEL_HESTON ? 2 : 1; }
};

Model to_model(const kx_model *m) {
    if (!m) fail(KX_INVALID_ARGUMENT, "null model");
    Model o;
    o.kind = m->kind;
    o.scheme = m->heston_scheme;
    o.s0 = m->s0; o.mu = m->mu; o.sigma = m->sigma;
    o.v0 = m->v0; o.kappa = m->kappa; o.theta = m->theta; o.sigma_v = m->sigma_v; o.rho = m->rho; o.r = m->r;
    if (m->asset) o.asset = m->asset;
    if (o.kind != KX_MODEL_GBM && o.kind != KX_MODEL_HESTON) fail(KX_INVALID_ARGUMENT, "unknown model kind");
    return o;
}

// simulator.rs:413-428
void validate_grid(const std::vector<double> &times) {
    if (times.empty()) fail(KX_INCONSISTENT_PATH, "empty grid");
    double prev = 0.0;
    for (double t : times) {
        if (t < prev) fail(KX_INCONSISTENT_PATH, "grid not increasing");
        prev = t;
    }
}

void validate_model(const Model &m) {
    if (m.kind == KX_MODEL_GBM) {
        if (m.sigma < 0.0) fail(KX_MALFORMED_CONTRACT, "GBM sigma must be non-negative");  // simulator.rs:221-225
    } else {  // simulator.rs:556-580
        if (!(m.rho >= -1.0 && m.rho <= 1.0)) fail(KX_MALFORMED_CONTRACT, "Heston rho must be in [-1, 1]");
        if (m.v0 < 0.0) fail(KX_MALFORMED_CONTRACT, "Heston v0 must be non-negative");
        if (m.sigma_v < 0.0) fail(KX_MALFORMED_CONTRACT, "Heston sigma_v must be non-negative");
        if (m.theta < 0.0) fail(KX_MALFORMED_CONTRACT, "Heston theta must be non-negative");
        if (m.kappa < 0.0) fail(KX_MALFORMED_CONTRACT, "Heston kappa must be non-negative");
    }
}

// One path on `times`; `z` holds the path's normals in draw order.
// GBM: simulator.rs:236-249. Heston: simulator.rs:506-541 (reference floor) or
// full truncation (Lord et al. 2010) when m.scheme says so.
void simulate_path(const Model &m, const std::vector<double> &times, const double *z, double *row) {
    size_t d = 0;
    double prev_t = 0.0;
    if (m.kind == KX_MODEL_GBM) {
        double s = m.s0;
        for (size_t k = 0; k < times.size(); ++k) {
            double t = times[k];
            double dt = t - prev_t;
            if (dt > 0.0) {
                double zz = z[d++];
                double drift = (m.mu - 0.5 * m.sigma * m.sigma) * dt;
                double diffusion = m.sigma * std::sqrt(dt) * zz;
                s *= std::exp(drift + diffusion);
            }
            row[k] = s;
            prev_t = t;
        }
    } else {
        double rho_perp = std::sqrt(std::max(1.0 - m.rho * m.rho, 0.0));
        double s = m.s0;
        double v = std::max(m.v0, 0.0);
        for (size_t k = 0; k < times.size(); ++k) {
            double t = times[k];
            double dt = t - prev_t;
            if (dt > 0.0) {
                double sqrt_dt = std::sqrt(dt);
                double z1 = z[d++];
                double z2 = z[d++];
                double dw_s = z1 * sqrt_dt;
                double dw_v = (m.rho * z1 + rho_perp * z2) * sqrt_dt;
                if (m.scheme == KX_HESTON_FULL_TRUNCATION) {
                    double vp = std::max(v, 0.0);
                    double sqrt_v = std::sqrt(vp);
                    s *= std::exp(m.r * dt - 0.5 * vp * dt + sqrt_v * dw_s);
                    v = v + m.kappa * (m.theta - vp) * dt + m.sigma_v * sqrt_v * dw_v;
                } else {
                    double sqrt_v = std::sqrt(v);
                    s *= std::exp(m.r * dt - 0.5 * v * dt + sqrt_v * dw_s);
                    double nv = v + m.kappa * (m.theta - v) * dt + m.sigma_v * sqrt_v * dw_v;
                    v = std::isnan(nv) ? 0.0 : std::max(nv, 0.0);  // f64::max(NaN, 0) = 0
                }
            }
            row[k] = s;
            prev_t = t;
        }
    }
}

size_t n_draws_for(const Model &m, const std::vector<double> &times) {
    size_t n = 0;
    double prev = 0.0;
    for (double t : times) { if (t - prev > 0.0) ++n; prev = t; }
    return n * m.draws_per_step();
}

// ---------------------------------------------------------------------------
// Path evaluation (src/observable.rs:92-168, src/pricer.rs:344-433)
// ---------------------------------------------------------------------------
struct PathView {
    const std::vector<double> *times;
    const double *spots;
    const std::string *asset;
    // a multi-asset path (Path::with_asset per factor): names[i]'s spots in rows[i]
    const std::vector<std::string> *names = nullptr;
    const double *const *rows = nullptr;
    size_t len() const { return times->size(); }
};

double eval_obs(const Obs &o, const PathView &p, size_t t);

double fmax_rs(double a, double b) { return std::fmax(a, b); }  // f64::max ignores NaN
double fmin_rs(double a, double b) { return std::fmin(a, b); }

double eval_obs(const Obs &o, const PathView &p, size_t t) {
    switch (o.k) {
    case O_CONST: return o.c;
    case O_SPOT:  // observable.rs:79-87
        if (p.names) {
            size_t i = 0;
            while (i < p.names->size() && (*p.names)[i] != o.name) ++i;
            if (i == p.names->size()) fail(KX_UNKNOWN_ASSET, o.name);
            if (t >= p.len()) fail(KX_STEP_OUT_OF_RANGE, std::to_string(t));
            return p.rows[i][t];
        }
        if (o.name != *p.asset) fail(KX_UNKNOWN_ASSET, o.name);
        if (t >= p.len()) fail(KX_STEP_OUT_OF_RANGE, std::to_string(t));
        return p.spots[t];
    case O_NEG: return -eval_obs(*o.a, p, t);
    case O_ADD: { double a = eval_obs(*o.a, p, t); return a + eval_obs(*o.b, p, t); }
    case O_SUB: { double a = eval_obs(*o.a, p, t); return a - eval_obs(*o.b, p, t); }
    case O_MUL: { double a = eval_obs(*o.a, p, t); return a * eval_obs(*o.b, p, t); }
    case O_DIV: { double a = eval_obs(*o.a, p, t); return a / eval_obs(*o.b, p, t); }
    case O_MAX: { double a = eval_obs(*o.a, p, t); return fmax_rs(a, eval_obs(*o.b, p, t)); }
    case O_MIN: { double a = eval_obs(*o.a, p, t); return fmin_rs(a, eval_obs(*o.b, p, t)); }
    case O_AVG: {  // observable.rs:103-134
        if (t >= p.len()) fail(KX_STEP_OUT_OF_RANGE, std::to_string(t));
        double t_now = (*p.times)[t];
        double t_from = o.has_from ? o.from : 0.0;
        double t_to = o.has_to ? o.to : t_now;
        if (t_from > t_to + 1e-12) fail(KX_MALFORMED_CONTRACT, "inverted average window");
        double sum = 0.0;
        size_t cnt = 0;
        for (size_t i = 0; i < p.len(); ++i) {
            double ti = (*p.times)[i];
            if (ti >= t_from - 1e-12 && ti <= t_to + 1e-12) { sum += eval_obs(*o.a, p, i); ++cnt; }
        }
        if (cnt == 0) fail(KX_MALFORMED_CONTRACT, "empty average window");
        return sum / (double)cnt;
    }
    case O_RMAX: {  // observable.rs:135-137
        double acc = -INFINITY;
        for (size_t i = 0; i <= t; ++i) acc = fmax_rs(acc, eval_obs(*o.a, p, i));
        return acc;
    }
    case O_RMIN: {
        double acc = INFINITY;
        for (size_t i = 0; i <= t; ++i) acc = fmin_rs(acc, eval_obs(*o.a, p, i));
        return acc;
    }
    }
    return 0.0;
}

bool eval_cond(const Cond &c, const PathView &p, size_t t) {  // observable.rs:150-168
    switch (c.k) {
    case C_BOOL: return c.b;
    case C_AT:
        if (t >= p.len()) fail(KX_STEP_OUT_OF_RANGE, std::to_string(t));
        return (*p.times)[t] + 1e-12 >= c.t;
    case C_GE: { double a = eval_obs(*c.l, p, t); return a >= eval_obs(*c.r, p, t); }
    case C_GT: { double a = eval_obs(*c.l, p, t); return a > eval_obs(*c.r, p, t); }
    case C_LE: { double a = eval_obs(*c.l, p, t); return a <= eval_obs(*c.r, p, t); }
    case C_LT: { double a = eval_obs(*c.l, p, t); return a < eval_obs(*c.r, p, t); }
    case C_AND: return eval_cond(*c.x, p, t) && eval_cond(*c.y, p, t);
    case C_OR: return eval_cond(*c.x, p, t) || eval_cond(*c.y, p, t);
    case C_NOT: return !eval_cond(*c.x, p, t);
    }
    return false;
}

// pricer.rs:421-433
long first_activation(const Cond &c, const PathView &p, size_t start) {
    for (size_t t = start; t < p.len(); ++t)
        if (eval_cond(c, p, t)) return (long)t;
    return -1;
}

using Flows = std::vector<std::pair<double, size_t>>;

// pricer.rs:374-418
void cashflows(const Con &c, size_t t_idx, const PathView &p, Flows &out) {
    switch (c.k) {
    case K_ZERO: return;
    case K_ONE: out.emplace_back(1.0, t_idx); return;
    case K_GIVE: {
        size_t s = out.size();
        cashflows(*c.a, t_idx, p, out);
        for (size_t i = s; i < out.size(); ++i) out[i].first = -out[i].first;
        return;
    }
    case K_AND: cashflows(*c.a, t_idx, p, out); cashflows(*c.b, t_idx, p, out); return;
    case K_SCALE: {
        size_t s = out.size();
        cashflows(*c.a, t_idx, p, out);
        for (size_t i = s; i < out.size(); ++i) out[i].first = out[i].first * eval_obs(*c.obs, p, out[i].second);
        return;
    }
    case K_WHEN: case K_ANYTIME: {
        long k = first_activation(*c.cond, p, t_idx);
        if (k >= 0) cashflows(*c.a, (size_t)k, p, out);
        return;
    }
    case K_UNTIL: {
        size_t s = out.size();
        cashflows(*c.a, t_idx, p, out);
        long k = first_activation(*c.cond, p, t_idx);
        if (k >= 0) {
            size_t w = s;
            for (size_t i = s; i < out.size(); ++i)
                if (out[i].second < (size_t)k) out[w++] = out[i];
            out.resize(w);
        }
        return;
    }
    case K_OR: fail(KX_UNSUPPORTED, "or (optimal choice needs LSM)");
    }
}

// pricer.rs:344-355
double present_value(const Con &c, const PathView &p, const std::vector<double> &grid, double rate) {
    Flows f;
    cashflows(c, 0, p, f);
    double s = 0.0;
    for (auto &fl : f) s += fl.first * std::exp(-rate * grid[fl.second]);
    return s;
}

// pricer.rs:303-328
kx_price_result summarize(const std::vector<double> &pvs) {
    const double Z95 = 1.959963984540054;
    size_t n = pvs.size();
    double sum = 0.0;
    for (double x : pvs) sum += x;
    double price = sum / (double)std::max<size_t>(n, 1);
    double sd = 0.0;
    if (n > 1) {
        double ss = 0.0;
        for (double x : pvs) ss += (x - price) * (x - price);
        sd = std::sqrt(ss / ((double)n - 1.0));
    }
    double se = n > 0 ? sd / std::sqrt((double)n) : 0.0;
    kx_price_result r;
    r.price = price;
    r.sample_std = sd;
    r.std_error = se;
    r.ci95_low = price - Z95 * se;
    r.ci95_high = price + Z95 * se;
    r.n_paths = n;
    return r;
}

// ---------------------------------------------------------------------------
// Drivers
// ---------------------------------------------------------------------------
struct SharedDraws {
    std::vector<double> z;
    uint64_t n_paths = 0, dpp = 0;
} g_shared;

int g_threads = 0;

NormalSource make_source(const kx_mc_config &cfg) {
    NormalSource ns;
    ns.seed = cfg.seed;
    if (cfg.rng == KX_RNG_SHARED_DRAWS) {
        if (g_shared.z.empty()) fail(KX_INVALID_ARGUMENT, "no shared draws registered");
        ns.shared = g_shared.z.data();
        ns.shared_paths = g_shared.n_paths;
        ns.shared_dpp = g_shared.dpp;
    } else if (cfg.rng != KX_RNG_PHILOX) {
        fail(KX_INVALID_ARGUMENT, "unknown rng");
    }
    return ns;
}

// Value `n_paths` paths of `model` on `grid` with each contract in `cons`;
// pvs[c][i]. Paths are materialised chunk by chunk (the reference keeps all of
// them; values per path are the same).
// negate: the antithetic paths (simulate_antithetic_gbm, variance_reduction.rs:76-129,
// whose anti path steps with drift - diff_scale * z, i.e. the normals negated).
void value_paths(const std::vector<const Con *> &cons, const Model &m, const std::vector<double> &grid,
                 uint64_t n_paths, const NormalSource &ns, double rate, std::vector<std::vector<double>> &pvs,
                 bool negate = false) {
    validate_model(m);
    validate_grid(grid);
    pvs.assign(cons.size(), std::vector<double>(n_paths));
    const size_t nd = n_draws_for(m, grid);
    const size_t chunk = 4096;
    int err_code = 0;
    std::string err_msg;
#pragma omp parallel num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
    {
        std::vector<double> rows(chunk * grid.size());
        std::vector<double> z(std::max<size_t>(nd, 1));
#pragma omp for schedule(dynamic, 1)
        for (int64_t c0 = 0; c0 < (int64_t)n_paths; c0 += (int64_t)chunk) {
            if (err_code) continue;
            try {
                uint64_t c1 = std::min<uint64_t>(n_paths, (uint64_t)c0 + chunk);
                // simulate (materialise) the chunk
                for (uint64_t i = (uint64_t)c0; i < c1; ++i) {
                    ns.fill(i, nd, z.data());
                    if (negate)
                        for (size_t q = 0; q < nd; ++q) z[q] = -z[q];
                    simulate_path(m, grid, z.data(), &rows[(i - c0) * grid.size()]);
                }
                // then value every path of the chunk
                for (size_t ci = 0; ci < cons.size(); ++ci)
                    for (uint64_t i = (uint64_t)c0; i < c1; ++i) {
                        PathView pv{&grid, &rows[(i - c0) * grid.size()], &m.asset};
                        pvs[ci][i] = present_value(*cons[ci], pv, grid, rate);
                    }
            } catch (const KxError &e) {
#pragma omp critical
                if (!err_code) { err_code = e.code; err_msg = e.msg; }
            }
        }
    }
    if (err_code) fail(err_code, err_msg);
}

kx_mc_config check_cfg(const kx_mc_config *cfg) {
    if (!cfg) fail(KX_INVALID_ARGUMENT, "null config");
    return *cfg;
}

int run(const std::function<void()> &f) {
    try {
        f();
        g_last_error.clear();
        return KX_OK;
    } catch (const KxError &e) {
        g_last_error = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return KX_INVALID_ARGUMENT;
    }
}

// numerics.rs:22-41 (Abramowitz-Stegun 7.1.26 erfc form)
double norm_cdf_as(double x) {
    double y = x / M_SQRT2;
    double sign = y < 0.0 ? -1.0 : 1.0;
    double xa = std::fabs(y);
    double t = 1.0 / (1.0 + 0.3275911 * xa);
    double poly = ((((1.061405429 * t - 1.453152027) * t) + 1.421413741) * t - 0.284496736) * t + 0.254829592;
    double erf_abs = 1.0 - poly * t * std::exp(-xa * xa);
    return 0.5 * (1.0 + sign * erf_abs);
}
double norm_cdf_exact(double x) { return 0.5 * std::erfc(-x / M_SQRT2); }

// numerics.rs:190-236 — Gauss elimination with partial pivoting; a pivot
// below 1e-12 returns the zero vector.
std::vector<double> solve_linear(std::vector<std::vector<double>> a, std::vector<double> b) {
    size_t n = b.size();
    for (size_t col = 0; col < n; ++col) {
        size_t piv = col;
        double best = std::fabs(a[col][col]);
        for (size_t row = col + 1; row < n; ++row) {
            double v = std::fabs(a[row][col]);
            if (v > best) { best = v; piv = row; }
        }
        if (best < 1e-12) return std::vector<double>(n, 0.0);
        std::swap(a[col], a[piv]);
        std::swap(b[col], b[piv]);
        for (size_t row = col + 1; row < n; ++row) {
            double factor = a[row][col] / a[col][col];
            for (size_t c = col; c < n; ++c) a[row][c] -= factor * a[col][c];
            b[row] -= factor * b[col];
        }
    }
    std::vector<double> x(n, 0.0);
    for (size_t row = n; row-- > 0;) {
        double sum = b[row];
        for (size_t c = row + 1; c < n; ++c) sum -= a[row][c] * x[c];
        x[row] = sum / a[row][row];
    }
    return x;
}

// lsm.rs:259-288 — normal equations of the monomial basis over (xs, ys).
std::vector<double> poly_fit(const std::vector<double> &xs, const std::vector<double> &ys, size_t m) {
    std::vector<std::vector<double>> ata(m, std::vector<double>(m, 0.0));
    std::vector<double> aty(m, 0.0), pw(m, 1.0);
    for (size_t k = 0; k < xs.size(); ++k) {
        pw[0] = 1.0;
        for (size_t j = 1; j < m; ++j) pw[j] = pw[j - 1] * xs[k];
        for (size_t r = 0; r < m; ++r) {
            aty[r] += pw[r] * ys[k];
            for (size_t c = 0; c < m; ++c) ata[r][c] += pw[r] * pw[c];
        }
    }
    return solve_linear(ata, aty);
}
// Weighted Laguerre basis e^(-x/2) L_j(x), x = s / x_scale, j < m (an extra
// mode; the reference regresses on monomials only): L_0 = 1, L_1 = 1 - x,
// (j + 1) L_(j+1) = (2j + 1 - x) L_j - j L_(j-1).
void laguerre_basis(double s, double x_scale, size_t m, std::vector<double> &phi) {
    const double x = s / x_scale;
    const double w = std::exp(-0.5 * x);
    double lm = 1.0, l = 1.0 - x;
    phi[0] = w;
    if (m > 1) phi[1] = w * l;
    for (size_t j = 1; j + 1 < m; ++j) {
        const double ln = ((double)(2 * j + 1) - x) * l - (double)j * lm;
        const double lnn = ln / (double)(j + 1);
        lm = l;
        l = lnn;
        phi[j + 1] = w * l;
    }
}
std::vector<double> laguerre_fit(const std::vector<double> &xs, const std::vector<double> &ys, size_t m,
                                 double x_scale) {
    std::vector<std::vector<double>> ata(m, std::vector<double>(m, 0.0));
    std::vector<double> aty(m, 0.0), phi(m);
    for (size_t k = 0; k < xs.size(); ++k) {
        laguerre_basis(xs[k], x_scale, m, phi);
        for (size_t r = 0; r < m; ++r) {
            aty[r] += phi[r] * ys[k];
            for (size_t c = 0; c < m; ++c) ata[r][c] += phi[r] * phi[c];
        }
    }
    return solve_linear(ata, aty);
}
double laguerre_eval(const std::vector<double> &c, double s, double x_scale) {
    std::vector<double> phi(c.size());
    laguerre_basis(s, x_scale, c.size(), phi);
    double acc = 0.0;
    for (size_t j = 0; j < c.size(); ++j) acc += c[j] * phi[j];
    return acc;
}

double poly_eval(const std::vector<double> &c, double x) {  // lsm.rs:293-295
    double acc = 0.0;
    for (size_t i = c.size(); i-- > 0;) acc = acc * x + c[i];
    return acc;
}

}  // namespace

// ===========================================================================
// C API of the oracle (ctypes; test infrastructure only)
// ===========================================================================
extern "C" {

const char *ko_last_error(void) { return g_last_error.c_str(); }

void ko_set_threads(int n) { g_threads = n; }

int ko_max_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

int ko_set_shared_draws(const double *z, uint64_t n_paths, uint64_t dpp) {
    return run([&] {
        if (!z && (n_paths * dpp) != 0) fail(KX_INVALID_ARGUMENT, "null draws");
        g_shared.z.assign(z, z + n_paths * dpp);
        g_shared.n_paths = n_paths;
        g_shared.dpp = dpp;
    });
}

// JSON parse check: returns KX_OK or the Serde/Unsupported status.
int ko_parse(const char *json) {
    return run([&] { parse_contract(json); });
}

// Plan (compiler.rs:25-34); assets separated by '\n'.
int ko_plan(const char *json, kx_plan_info *info, double *dates, size_t cap, char *assets, size_t acap) {
    return run([&] {
        ConP c = parse_contract(json);
        Plan p = compile(*c);
        info->n_assets = (uint32_t)p.assets.size();
        info->n_fixed_dates = (uint32_t)p.fixed_dates.size();
        info->horizon = p.horizon;
        info->needs_fine_grid = p.needs_fine;
        info->n_triggers = info->n_flows = info->n_accumulators = 0;
        for (size_t i = 0; i < p.fixed_dates.size() && i < cap; ++i) dates[i] = p.fixed_dates[i];
        std::string s;
        for (size_t i = 0; i < p.assets.size(); ++i) { if (i) s += '\n'; s += p.assets[i]; }
        if (assets && acap) { strncpy(assets, s.c_str(), acap - 1); assets[acap - 1] = 0; }
    });
}

int ko_time_grid(const char *json, uint32_t spy, int force, double *out, size_t cap, size_t *n) {
    return run([&] {
        ConP c = parse_contract(json);
        auto g = time_grid_forced(compile(*c), spy, force != 0);
        *n = g.size();
        for (size_t i = 0; i < g.size() && i < cap; ++i) out[i] = g[i];
    });
}

// Gbm::simulate / HestonSimulator::simulate on an explicit grid: out[i*n_grid+k].
int ko_simulate(const kx_model *model, const double *grid, size_t n_grid, uint64_t n_paths,
                const kx_mc_config *cfg, double *out) {
    return run([&] {
        Model m = to_model(model);
        validate_model(m);
        std::vector<double> g(grid, grid + n_grid);
        validate_grid(g);
        NormalSource ns = make_source(check_cfg(cfg));
        size_t nd = n_draws_for(m, g);
#pragma omp parallel for num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
        for (int64_t i = 0; i < (int64_t)n_paths; ++i) {
            std::vector<double> z(std::max<size_t>(nd, 1));
            ns.fill((uint64_t)i, nd, z.data());
            simulate_path(m, g, z.data(), out + (size_t)i * n_grid);
        }
    });
}

// Normals of one path (for tests of the Philox stream).
int ko_normals(uint64_t seed, uint64_t path, size_t n, double *out) {
    return run([&] {
        NormalSource ns;
        ns.seed = seed;
        ns.fill(path, n, out);
    });
}

// price_gbm (pricer.rs:97-115) without variance reduction.
int ko_price(const char *json, const kx_model *model, const kx_mc_config *cfg, kx_price_result *out,
             double *per_path) {
    return run([&] {
        ConP c = parse_contract(json);
        Model m = to_model(model);
        kx_mc_config mc = check_cfg(cfg);
        Plan p = compile(*c);
        auto grid = time_grid_forced(p, mc.steps_per_year, m.requires_fine());
        std::vector<std::vector<double>> pvs;
        value_paths({c.get()}, m, grid, mc.n_paths, make_source(mc), mc.rate, pvs);
        *out = summarize(pvs[0]);
        if (per_path) memcpy(per_path, pvs[0].data(), pvs[0].size() * sizeof(double));
    });
}

double ko_bs_call(double s, double k, double t, double r, double sigma);

// price_gbm with variance reduction (pricer.rs:108-230, variance_reduction.rs:60-235).
// flags: 1 antithetic, 2 control variate (the ATM call at the grid's last date).
int ko_price_vr(const char *json, const kx_model *model, const kx_mc_config *cfg, int flags, kx_price_result *out) {
    return run([&] {
        ConP c = parse_contract(json);
        Model m = to_model(model);
        kx_mc_config mc = check_cfg(cfg);
        Plan p = compile(*c);
        auto grid = time_grid_forced(p, mc.steps_per_year, m.requires_fine());
        const bool gbm = m.kind == KX_MODEL_GBM;
        const bool anti = (flags & 1) && gbm;  // Simulator::simulate_antithetic_paths: None unless GBM
        const bool cv = (flags & 2) != 0;
        const double s0 = gbm ? m.s0 : 100.0, sigma = gbm ? m.sigma : 0.2;  // gbm_params().unwrap_or
        const double t_mat = grid.empty() ? 1.0 : grid.back();
        ConP ctrl;
        double bs = 0.0;
        if (cv) {  // pricer.rs:160-167
            char buf[512];
            snprintf(buf, sizeof buf,
                     "{\"When\":[{\"At\":%.17g},{\"Scale\":[{\"Max\":[{\"Sub\":[{\"Spot\":\"%s\"},{\"Const\":%.17g}]},"
                     "{\"Const\":0.0}]},{\"One\":\"USD\"}]}]}",
                     t_mat, m.asset.c_str(), s0);
            ctrl = parse_contract(buf);
            bs = ko_bs_call(s0, s0, t_mat, mc.rate, sigma);
        }
        const NormalSource ns = make_source(mc);
        std::vector<const Con *> cons{c.get()};
        if (cv) cons.push_back(ctrl.get());
        if (anti) {
            const uint64_t n_half = mc.n_paths / 2;
            std::vector<std::vector<double>> b, a;
            value_paths(cons, m, grid, n_half, ns, mc.rate, b);
            value_paths(cons, m, grid, n_half, ns, mc.rate, a, true);
            auto pairs = [&](size_t q) {  // price_antithetic_on_paths
                std::vector<double> v(n_half);
                for (uint64_t i = 0; i < n_half; ++i) v[i] = 0.5 * (b[q][i] + a[q][i]);
                return summarize(v);
            };
            if (!cv) {
                *out = pairs(0);
                return;
            }
            const kx_price_result res = pairs(0), ctl = pairs(1);  // price_antithetic_with_cv
            kx_price_result r{};
            r.price = res.price - 1.0 * (ctl.price - bs);
            const uint64_t n = 2 * n_half;
            r.sample_std = res.sample_std;
            r.std_error = res.sample_std / std::sqrt((double)n);
            r.ci95_low = r.price - 1.959963984540054 * r.std_error;
            r.ci95_high = r.price + 1.959963984540054 * r.std_error;
            r.n_paths = n;
            *out = r;
            return;
        }
        std::vector<std::vector<double>> pvs;
        value_paths(cons, m, grid, mc.n_paths, ns, mc.rate, pvs);
        if (cv) {  // price_control_variate_on_paths with beta = 1
            for (uint64_t i = 0; i < mc.n_paths; ++i) pvs[0][i] = pvs[0][i] - 1.0 * (pvs[1][i] - bs);
        }
        *out = summarize(pvs[0]);
    });
}

// price_on_paths over an explicit grid (pricer.rs:230-241): the grid is given
// by the caller instead of the compiler (used by tests of Heston on a fixed grid).
int ko_price_on_grid(const char *json, const kx_model *model, const kx_mc_config *cfg, const double *grid,
                     size_t n_grid, kx_price_result *out) {
    return run([&] {
        ConP c = parse_contract(json);
        Model m = to_model(model);
        kx_mc_config mc = check_cfg(cfg);
        std::vector<double> g(grid, grid + n_grid);
        std::vector<std::vector<double>> pvs;
        value_paths({c.get()}, m, g, mc.n_paths, make_source(mc), mc.rate, pvs);
        *out = summarize(pvs[0]);
    });
}

// price_batch_gbm (pricer.rs:250-294).
int ko_price_batch(size_t n, const char *const *jsons, const kx_model *model, const kx_mc_config *cfg,
                   kx_price_result *out) {
    return run([&] {
        if (n == 0) return;
        std::vector<ConP> cons;
        Plan merged;
        for (size_t i = 0; i < n; ++i) {
            cons.push_back(parse_contract(jsons[i]));
            Plan p = compile(*cons.back());
            merged.fixed_dates.insert(merged.fixed_dates.end(), p.fixed_dates.begin(), p.fixed_dates.end());
            merged.horizon = std::max(merged.horizon, p.horizon);
            merged.needs_fine = merged.needs_fine | p.needs_fine;
        }
        Model m = to_model(model);
        kx_mc_config mc = check_cfg(cfg);
        auto grid = time_grid_forced(merged, mc.steps_per_year, m.requires_fine());
        std::vector<const Con *> raw;
        for (auto &c : cons) raw.push_back(c.get());
        std::vector<std::vector<double>> pvs;
        value_paths(raw, m, grid, mc.n_paths, make_source(mc), mc.rate, pvs);
        for (size_t i = 0; i < n; ++i) out[i] = summarize(pvs[i]);
    });
}

// greeks_gbm (greeks.rs:60-98): 7 reprices with the same normals. Bumps are
// absolute, or relative to the bumped value when bumps->relative != 0.
// greeks_gbm (greeks.rs:60-98) of contract c at spot s0 and volatility sigma:
// seven reprices on the same normals, price / delta / gamma from the spot
// reprices, vega and rho from the vol and rate ones, each a difference of
// means; the standard errors are those of the per-path differences.
static void greeks_at(const ConP &c, const Model &base, const kx_mc_config &mc, const kx_bumps &b, double s0,
                      double sigma, kx_greeks *out) {
    double r = mc.rate;
    double hs = b.relative ? b.spot * s0 : b.spot;
    double hv = b.relative ? b.vol * sigma : b.vol;
    double hr = b.relative ? b.rate * r : b.rate;
    Plan p = compile(*c);
    auto grid = time_grid_forced(p, mc.steps_per_year, false);
    NormalSource ns = make_source(mc);
    auto reprice = [&](double s, double sg, double rate, std::vector<double> &pv) {
        Model m = base;
        m.s0 = s; m.mu = rate; m.sigma = sg;  // Gbm::new(asset, s0, rate, sigma), greeks.rs:70
        std::vector<std::vector<double>> pvs;
        value_paths({c.get()}, m, grid, mc.n_paths, ns, rate, pvs);
        pv = std::move(pvs[0]);
    };
    std::vector<double> p0, psu, psd, pvu, pvd, pru, prd;
    reprice(s0, sigma, r, p0);
    reprice(s0 + hs, sigma, r, psu);
    reprice(s0 - hs, sigma, r, psd);
    reprice(s0, sigma + hv, r, pvu);
    reprice(s0, sigma - hv, r, pvd);
    reprice(s0, sigma, r + hr, pru);
    reprice(s0, sigma, r - hr, prd);
    auto mean = [](const std::vector<double> &v) { return summarize(v).price; };
    double price = mean(p0), su = mean(psu), sd = mean(psd);
    out->price = price;
    out->delta = (su - sd) / (2.0 * hs);
    out->gamma = (su - 2.0 * price + sd) / (hs * hs);
    out->vega = (mean(pvu) - mean(pvd)) / (2.0 * hv);
    out->rho = (mean(pru) - mean(prd)) / (2.0 * hr);
    size_t n = p0.size();
    std::vector<double> e(n);
    auto se_of = [&](auto f) { for (size_t i = 0; i < n; ++i) e[i] = f(i); return summarize(e).std_error; };
    out->price_se = summarize(p0).std_error;
    out->delta_se = se_of([&](size_t i) { return (psu[i] - psd[i]) / (2.0 * hs); });
    out->gamma_se = se_of([&](size_t i) { return (psu[i] - 2.0 * p0[i] + psd[i]) / (hs * hs); });
    out->vega_se = se_of([&](size_t i) { return (pvu[i] - pvd[i]) / (2.0 * hv); });
    out->rho_se = se_of([&](size_t i) { return (pru[i] - prd[i]) / (2.0 * hr); });
}

int ko_greeks(const char *json, const kx_model *model, const kx_mc_config *cfg, const kx_bumps *bumps,
              kx_greeks *out) {
    return run([&] {
        ConP c = parse_contract(json);
        Model base = to_model(model);
        if (base.kind != KX_MODEL_GBM) fail(KX_UNSUPPORTED, "greeks need a GBM model");
        kx_mc_config mc = check_cfg(cfg);
        kx_bumps b = bumps ? *bumps : kx_bumps{1e-2, 1e-2, 1e-4, 0, 0, 0.0};
        greeks_at(c, base, mc, b, base.s0, base.sigma, out);
    });
}

// greek_surface (surface.rs:104-137): greeks_gbm at every (spots[i], vols[j]),
// out[i * n_vols + j]; an empty grid is InconsistentPath (surface.rs:113-117).
int ko_greek_surface(const char *json, const char *asset, const double *spots, size_t n_spots, const double *vols,
                     size_t n_vols, const kx_mc_config *cfg, const kx_bumps *bumps, kx_greeks *out) {
    return run([&] {
        if (n_spots == 0 || n_vols == 0) fail(KX_INCONSISTENT_PATH, "empty surface grid");
        ConP c = parse_contract(json);
        kx_mc_config mc = check_cfg(cfg);
        kx_bumps b = bumps ? *bumps : kx_bumps{1e-2, 1e-2, 1e-4, 0, 0, 0.0};
        kx_model cm{};
        cm.kind = KX_MODEL_GBM;
        cm.s0 = spots[0];
        cm.mu = mc.rate;
        cm.sigma = vols[0];
        cm.asset = asset;
        Model base = to_model(&cm);
        for (size_t i = 0; i < n_spots; ++i)
            for (size_t j = 0; j < n_vols; ++j) greeks_at(c, base, mc, b, spots[i], vols[j], &out[i * n_vols + j]);
    });
}

// price_gbm of one contract under `m`, or false where the reference's
// price_gbm returns an error (the calibration objectives skip those quotes).
static bool try_price(const ConP &c, const Model &m, const kx_mc_config &mc, double &price) {
    try {
        Plan p = compile(*c);
        auto grid = time_grid_forced(p, mc.steps_per_year, m.requires_fine());
        std::vector<std::vector<double>> pvs;
        value_paths({c.get()}, m, grid, mc.n_paths, make_source(mc), mc.rate, pvs);
        price = summarize(pvs[0]).price;
        return true;
    } catch (const KxError &) {
        return false;
    }
}

// gbm_prices (calibration.rs:72-90) for several volatilities:
// out[k * n_quotes + i] under Gbm::new(asset, spots[i], rate, sigmas[k]), NaN on error.
int ko_calib_gbm_prices(const char *json, const char *asset, const double *spots, size_t n_quotes,
                        const double *sigmas, size_t n_sigmas, const kx_mc_config *cfg, double *out) {
    return run([&] {
        ConP c = parse_contract(json);
        kx_mc_config mc = check_cfg(cfg);
        for (size_t k = 0; k < n_sigmas; ++k)
            for (size_t i = 0; i < n_quotes; ++i) {
                kx_model cm{};
                cm.kind = KX_MODEL_GBM;
                cm.s0 = spots[i];
                cm.mu = mc.rate;
                cm.sigma = sigmas[k];
                cm.asset = asset;
                double p = 0.0;
                out[k * n_quotes + i] = try_price(c, to_model(&cm), mc, p) ? p : std::nan("");
            }
    });
}

// eval_obj_heston (calibration.rs:103-126) for each parameter vector
// (v0, kappa, theta, sigma_v, rho): the squared errors of the quotes that
// price, summed in quote order, over the number of quotes.
int ko_calib_heston_objective(const char *json, const char *asset, const double *quotes, size_t n_quotes,
                              const double *params, size_t n_params, const kx_mc_config *cfg, double *obj) {
    return run([&] {
        ConP c = parse_contract(json);
        kx_mc_config mc = check_cfg(cfg);
        for (size_t k = 0; k < n_params; ++k) {
            double sum = 0.0;
            for (size_t i = 0; i < n_quotes; ++i) {
                kx_model cm{};
                cm.kind = KX_MODEL_HESTON;
                cm.heston_scheme = KX_HESTON_REFERENCE_FLOOR;
                cm.s0 = quotes[2 * i];
                cm.v0 = params[5 * k];
                cm.kappa = params[5 * k + 1];
                cm.theta = params[5 * k + 2];
                cm.sigma_v = params[5 * k + 3];
                cm.rho = params[5 * k + 4];
                cm.r = mc.rate;
                cm.asset = asset;
                double p = 0.0;
                if (!try_price(c, to_model(&cm), mc, p)) continue;
                const double d = p - quotes[2 * i + 1];
                sum += d * d;
            }
            obj[k] = sum / (double)n_quotes;
        }
    });
}

// ---- multilevel Monte Carlo (mlmc.rs) ---------------------------------------
static uint64_t mix(uint64_t seed, uint64_t index) { return seed ^ (index * 0x9E3779B97F4A7C15ull); }  // simulator.rs:431

static std::vector<double> uniform_grid(double t_max, uint64_t n_steps) {  // simulator.rs:181-184
    uint64_t n = std::max<uint64_t>(n_steps, 1);
    std::vector<double> g(n + 1);
    for (uint64_t k = 0; k <= n; ++k) g[k] = t_max * (double)k / (double)n;
    return g;
}

// simulate_level_pair (simulator.rs:321-409 GBM, 592-690 Heston) then
// level_samples (mlmc.rs:276-305): ys[i] = PV(fine path i) - PV(coarse path i),
// the coarse path stepping with the sum of two fine normals. `seed` is the
// level's seed mix(cfg.seed, level) (mlmc.rs:288); path i draws the Philox
// stream keyed by mix(seed, level + 1), where the reference seeds its path
// generator with mix(mix(seed, level + 1), i) (simulator.rs:345).
static void level_values(const Con &con, const Model &m, double t_max, uint32_t level, uint64_t n, uint64_t seed,
                         double rate, std::vector<double> &ys) {
    const uint64_t nf = 1ull << level;
    const bool coarse = level > 0;
    const uint64_t nc = coarse ? nf / 2 : 0;
    const std::vector<double> gf = uniform_grid(t_max, nf);
    const std::vector<double> gc = coarse ? uniform_grid(t_max, nc) : std::vector<double>();
    const double dt_f = t_max / (double)nf;
    const double sqrt_dt_f = std::sqrt(dt_f);
    NormalSource ns;
    ns.seed = mix(seed, (uint64_t)level + 1);
    const bool gbm = m.kind == KX_MODEL_GBM;
    const size_t dpp = (gbm ? 1 : 2) * nf;
    ys.assign(n, 0.0);
    const double rho_perp = std::sqrt(std::max(1.0 - m.rho * m.rho, 0.0));
    // Heston Euler step with the floor on v (simulator.rs:615-633)
    auto heston_row = [&](const std::vector<std::pair<double, double>> &incs, double dt, double *row) {
        const double sqrt_dt = std::sqrt(dt);
        double sp = m.s0, v = std::max(m.v0, 0.0);
        row[0] = sp;
        for (size_t k = 0; k < incs.size(); ++k) {
            const double sqrt_v = std::sqrt(v);
            const double dw_s = incs[k].first * sqrt_dt;
            const double dw_v = (m.rho * incs[k].first + rho_perp * incs[k].second) * sqrt_dt;
            sp *= std::exp(m.r * dt - 0.5 * v * dt + sqrt_v * dw_s);
            v = std::max(v + m.kappa * (m.theta - v) * dt + m.sigma_v * sqrt_v * dw_v, 0.0);
            row[k + 1] = sp;
        }
    };
    int err_code = 0;
    std::string err_msg;
#pragma omp parallel num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
    {
        std::vector<double> z(std::max<size_t>(dpp, 1)), rf(gf.size()), rc(std::max<size_t>(gc.size(), 1));
        std::vector<std::pair<double, double>> inc;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < (int64_t)n; ++i) {
            if (err_code) continue;
            try {
                ns.fill((uint64_t)i, dpp, z.data());
                if (gbm) {
                    const double drift_f = (m.mu - 0.5 * m.sigma * m.sigma) * dt_f;
                    double sp = m.s0;
                    rf[0] = sp;
                    for (uint64_t k = 0; k < nf; ++k) {
                        sp *= std::exp(drift_f + m.sigma * sqrt_dt_f * z[k]);
                        rf[k + 1] = sp;
                    }
                    if (coarse) {
                        const double dt_c = t_max / (double)nc;
                        const double drift_c = (m.mu - 0.5 * m.sigma * m.sigma) * dt_c;
                        sp = m.s0;
                        rc[0] = sp;
                        for (uint64_t j = 0; j < nc; ++j) {
                            const double dw = z[2 * j] + z[2 * j + 1];
                            sp *= std::exp(drift_c + m.sigma * sqrt_dt_f * dw);
                            rc[j + 1] = sp;
                        }
                    }
                } else {
                    inc.resize(nf);
                    for (uint64_t k = 0; k < nf; ++k) inc[k] = {z[2 * k], z[2 * k + 1]};
                    heston_row(inc, dt_f, rf.data());
                    if (coarse) {
                        const double inv_sqrt2 = 0.70710678118654752440;
                        std::vector<std::pair<double, double>> ic(nc);
                        for (uint64_t j = 0; j < nc; ++j)
                            ic[j] = {(inc[2 * j].first + inc[2 * j + 1].first) * inv_sqrt2,
                                     (inc[2 * j].second + inc[2 * j + 1].second) * inv_sqrt2};
                        heston_row(ic, t_max / (double)nc, rc.data());
                    }
                }
                PathView pf{&gf, rf.data(), &m.asset};
                const double vf = present_value(con, pf, gf, rate);
                double vc = 0.0;
                if (coarse) {
                    PathView pc{&gc, rc.data(), &m.asset};
                    vc = present_value(con, pc, gc, rate);
                }
                ys[(size_t)i] = vf - vc;
            } catch (const KxError &e) {
#pragma omp critical
                if (!err_code) { err_code = e.code; err_msg = e.msg; }
            }
        }
    }
    if (err_code) fail(err_code, err_msg);
}

// mean_var (mlmc.rs:318-332): two-pass mean and unbiased variance
static void mean_var(const std::vector<double> &xs, double &mean, double &var) {
    const size_t n = xs.size();
    mean = var = 0.0;
    if (n == 0) return;
    double s = 0.0;
    for (double x : xs) s += x;
    mean = s / (double)n;
    if (n > 1) {
        double q = 0.0;
        for (double x : xs) q += (x - mean) * (x - mean);
        var = q / ((double)n - 1.0);
    }
}

int ko_mlmc_level_values(const char *json, const kx_model *model, const kx_mc_config *cfg, uint32_t level,
                         uint64_t n, double *ys) {
    return run([&] {
        ConP c = parse_contract(json);
        Model m = to_model(model);
        kx_mc_config mc = check_cfg(cfg);
        validate_model(m);
        Plan p = compile(*c);
        std::vector<double> v;
        level_values(*c, m, p.horizon, level, n, mix(mc.seed, level), mc.rate, v);  // mlmc.rs:288
        memcpy(ys, v.data(), n * sizeof(double));
    });
}

// optimal_allocation (mlmc.rs:231-258)
static std::vector<uint64_t> optimal_allocation(const std::vector<double> &v, const std::vector<uint64_t> &c,
                                                double target) {
    const size_t l = std::min(v.size(), c.size());
    std::vector<uint64_t> out(l, 0);
    if (l == 0 || target <= 0.0) return out;
    double sum = 0.0;
    for (size_t k = 0; k < l; ++k) sum += std::sqrt(std::max(v[k], 0.0) * (double)std::max<uint64_t>(c[k], 1));
    for (size_t k = 0; k < l; ++k) {
        const double vk = std::max(v[k], 0.0), ck = (double)std::max<uint64_t>(c[k], 1);
        if (vk <= 0.0) {
            out[k] = 1;
            continue;
        }
        out[k] = std::max<uint64_t>((uint64_t)std::ceil((sum * std::sqrt(vk / ck)) / target), 1);
    }
    return out;
}

int ko_mlmc_optimal_allocation(const double *v, const uint64_t *c, size_t n, double target, uint64_t *out) {
    return run([&] {
        auto r = optimal_allocation(std::vector<double>(v, v + n), std::vector<uint64_t>(c, c + n), target);
        for (size_t k = 0; k < n; ++k) out[k] = r[k];
    });
}

// price_mlmc_detailed (mlmc.rs:107-215)
int ko_price_mlmc(const char *json, const kx_model *model, const kx_mc_config *cfg, const kx_mlmc_cfg *mcfg,
                  kx_mlmc_result *out) {
    return run([&] {
        ConP c = parse_contract(json);
        Model m = to_model(model);
        kx_mc_config mc = check_cfg(cfg);
        validate_model(m);
        const uint32_t L = mcfg->n_levels;
        if (L > KX_MLMC_MAX_LEVELS) fail(KX_INVALID_ARGUMENT, "too many levels");
        Plan p = compile(*c);
        const double t_max = p.horizon;
        std::vector<uint64_t> costs(L + 1);
        for (uint32_t l = 0; l <= L; ++l)
            costs[l] = (l == 0 ? 1 : (1ull << l) + (1ull << (l - 1))) * std::max<uint32_t>(mcfg->cost_per_step, 1);
        std::vector<double> means(L + 1, 0.0), var(L + 1, 0.0), sums(L + 1, 0.0), sumsq(L + 1, 0.0);
        std::vector<uint64_t> counts(L + 1, 0);
        std::vector<double> ys;
        for (uint32_t l = 0; l <= L; ++l) {
            ys.clear();
            if (mcfg->pilot_paths) level_values(*c, m, t_max, l, mcfg->pilot_paths, mix(mc.seed, l), mc.rate, ys);
            mean_var(ys, means[l], var[l]);
            for (double y : ys) sums[l] += y;
            for (double y : ys) sumsq[l] += y * y;
            counts[l] = ys.size();
        }
        auto extra = optimal_allocation(var, costs, mcfg->target_variance);
        const uint64_t seed_main = mc.seed ^ 0xA5A55A5ADEADBEEFull;
        for (uint32_t l = 0; l <= L; ++l) {
            if (extra[l] == 0) continue;
            level_values(*c, m, t_max, l, extra[l], mix(seed_main, l), mc.rate, ys);
            double s = 0.0, q = 0.0;
            for (double y : ys) s += y;
            for (double y : ys) q += y * y;
            sums[l] += s;
            sumsq[l] += q;
            counts[l] += ys.size();
        }
        memset(out, 0, sizeof *out);
        out->n_levels = L;
        double price = 0.0, var_q = 0.0;
        uint64_t n_total = 0, total_cost = 0;
        for (uint32_t l = 0; l <= L; ++l) {
            const double n = (double)std::max<uint64_t>(counts[l], 1);
            const double mean = sums[l] / n;
            const double v = counts[l] > 1 ? std::max((sumsq[l] - n * mean * mean) / (n - 1.0), 0.0) : 0.0;
            out->level_means[l] = mean;
            out->level_variances[l] = v;
            out->level_costs[l] = costs[l];
            out->level_paths[l] = counts[l];
            price += mean;
            var_q += v / n;
            n_total += counts[l];
            total_cost += counts[l] * costs[l];
        }
        const double se = std::sqrt(std::max(var_q, 0.0));
        const double Z95 = 1.959963984540054;
        out->price.price = price;
        out->price.std_error = se;
        out->price.sample_std = se * std::sqrt((double)std::max<uint64_t>(n_total, 1));
        out->price.ci95_low = price - Z95 * se;
        out->price.ci95_high = price + Z95 * se;
        out->price.n_paths = n_total;
        out->total_cost = total_cost;
    });
}

// ---- correlated multi-factor GBM (multi_asset.rs) ---------------------------
// numerics::cholesky_lower (numerics.rs:158-183)
static std::vector<std::vector<double>> cholesky_lower(const std::vector<std::vector<double>> &a) {
    const size_t n = a.size();
    std::vector<std::vector<double>> l(n, std::vector<double>(n, 0.0));
    for (size_t i = 0; i < n; ++i)
        for (size_t j = 0; j <= i; ++j) {
            double sum = a[i][j];
            for (size_t k = 0; k < j; ++k) sum -= l[i][k] * l[j][k];
            if (i == j) {
                l[i][j] = std::sqrt(std::max(sum, 0.0));
            } else {
                const double pivot = l[j][j];
                l[i][j] = pivot > 0.0 ? sum / pivot : 0.0;
            }
        }
    return l;
}

// price_gbm under CorrelatedGbmN::simulate_paths (multi_asset.rs:127-170): per
// grid step k >= 1 the normals (k - 1) n .. (k - 1) n + n - 1 of the path's
// Philox stream, w = L z, and every factor's exact step (evolve, :85-104).
int ko_price_multi(const char *json, const kx_multi_gbm *mm, const kx_mc_config *cfg, kx_price_result *out,
                   double *per_path) {
    return run([&] {
        ConP c = parse_contract(json);
        kx_mc_config mc = check_cfg(cfg);
        const size_t n = mm->n_assets;
        if (n < 2) fail(KX_MALFORMED_CONTRACT, "CorrelatedGbmN: at least 2 assets required");
        std::vector<std::string> names;
        std::vector<std::vector<double>> corr(n, std::vector<double>(n));
        for (size_t i = 0; i < n; ++i) {
            if (mm->sigma[i] < 0.0) fail(KX_MALFORMED_CONTRACT, "CorrelatedGbmN: every volatility must be >= 0");
            names.push_back(mm->names[i]);
            for (size_t j = 0; j < n; ++j) corr[i][j] = mm->corr[i * n + j];
        }
        const auto L = cholesky_lower(corr);
        Plan p = compile(*c);
        const auto grid = time_grid_forced(p, mc.steps_per_year, false);
        const size_t G = grid.size();
        NormalSource ns = make_source(mc);
        std::vector<double> pvs(mc.n_paths);
        int err_code = 0;
        std::string err_msg;
#pragma omp parallel num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
        {
            std::vector<double> z(std::max<size_t>((G - 1) * n, 1)), rows(n * G), w(n);
            std::vector<const double *> rp(n);
#pragma omp for schedule(dynamic, 256)
            for (int64_t i = 0; i < (int64_t)mc.n_paths; ++i) {
                if (err_code) continue;
                try {
                    ns.fill((uint64_t)i, (G - 1) * n, z.data());
                    std::vector<double> sp(mm->s0, mm->s0 + n);
                    for (size_t a = 0; a < n; ++a) rows[a * G] = sp[a];
                    double prev_t = grid[0];
                    for (size_t k = 1; k < G; ++k) {
                        const double dt = grid[k] - prev_t;
                        for (size_t a = 0; a < n; ++a) {
                            double acc = 0.0;
                            for (size_t j = 0; j <= a; ++j) acc += L[a][j] * z[(k - 1) * n + j];
                            w[a] = acc;
                        }
                        for (size_t a = 0; a < n; ++a) {
                            if (dt > 0.0)
                                sp[a] *= std::exp((mm->mu[a] - 0.5 * mm->sigma[a] * mm->sigma[a]) * dt +
                                                  mm->sigma[a] * std::sqrt(dt) * w[a]);
                            rows[a * G + k] = sp[a];
                        }
                        prev_t = grid[k];
                    }
                    for (size_t a = 0; a < n; ++a) rp[a] = &rows[a * G];
                    PathView pv{&grid, rows.data(), &names[0], &names, rp.data()};
                    pvs[(size_t)i] = present_value(*c, pv, grid, mc.rate);
                } catch (const KxError &e) {
#pragma omp critical
                    if (!err_code) { err_code = e.code; err_msg = e.msg; }
                }
            }
        }
        if (err_code) fail(err_code, err_msg);
        *out = summarize(pvs);
        if (per_path) memcpy(per_path, pvs.data(), pvs.size() * sizeof(double));
    });
}

// price_american_lsm (lsm.rs:80-229) with, per path (each array nullable, n
// entries): the discounted realised value (lsm.rs:226), the exercise date of
// the path (index into dates; -1 when the path is never exercised, i.e. its
// payoff is 0 at the last date and it was continued at every earlier one),
// and the decision margin: the smallest |exercise value - continuation| over
// the dates where the path was in the money and a regression decided
// (+inf when there was none). A decision can only differ between two
// implementations whose fitted continuations differ by more than its margin.
int ko_price_american_detail(const char *json, const kx_model *model, const kx_mc_config *cfg, const double *dates,
                             size_t n_dates, int n_basis, int basis, kx_price_result *out, double *per_path,
                             int32_t *ex_index, double *margin) {
    return run([&] {
        ConP c = parse_contract(json);
        Model m = to_model(model);
        kx_mc_config mc = check_cfg(cfg);
        if (n_dates == 0) fail(KX_MALFORMED_CONTRACT, "LSM: at least one exercise date");
        for (size_t i = 1; i < n_dates; ++i)
            if (dates[i] <= dates[i - 1]) fail(KX_MALFORMED_CONTRACT, "LSM: dates must increase and be > 0");
        if (dates[0] <= 0.0) fail(KX_MALFORMED_CONTRACT, "LSM: dates must increase and be > 0");
        if (n_basis < 2) fail(KX_MALFORMED_CONTRACT, "LSM: n_basis >= 2");
        validate_model(m);
        std::vector<double> grid{0.0};
        grid.insert(grid.end(), dates, dates + n_dates);
        const size_t G = grid.size(), np = mc.n_paths;
        NormalSource ns = make_source(mc);
        size_t nd = n_draws_for(m, grid);
        std::vector<double> paths(np * G);
#pragma omp parallel for num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
        for (int64_t i = 0; i < (int64_t)np; ++i) {
            std::vector<double> z(std::max<size_t>(nd, 1));
            ns.fill((uint64_t)i, nd, z.data());
            simulate_path(m, grid, z.data(), &paths[(size_t)i * G]);
        }
        const size_t n_ex = n_dates;
        // payoff[d][i] = value of the exercised contract at date index d+1 (lsm.rs:238-251)
        std::vector<std::vector<double>> payoff(n_ex, std::vector<double>(np)), spots(n_ex, std::vector<double>(np));
        int err = 0;
        std::string emsg;
#pragma omp parallel for num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
        for (int64_t i = 0; i < (int64_t)np; ++i) {
            try {
                PathView pv{&grid, &paths[(size_t)i * G], &m.asset};
                for (size_t d = 0; d < n_ex; ++d) {
                    size_t ti = d + 1;
                    double t_ex = grid[ti];
                    Flows f;
                    cashflows(*c, ti, pv, f);
                    double s = 0.0;
                    for (auto &fl : f) s += fl.first * std::exp(-mc.rate * (grid[fl.second] - t_ex));
                    payoff[d][(size_t)i] = s;
                    spots[d][(size_t)i] = paths[(size_t)i * G + ti];
                }
            } catch (const KxError &e) {
#pragma omp critical
                if (!err) { err = e.code; emsg = e.msg; }
            }
        }
        if (err) fail(err, emsg);
        // backward induction (lsm.rs:129-229)
        std::vector<double> value = payoff[n_ex - 1];
        std::vector<int32_t> exi(np);
        std::vector<double> mrg(np, std::numeric_limits<double>::infinity());
        for (size_t i = 0; i < np; ++i) exi[i] = payoff[n_ex - 1][i] > 0.0 ? (int32_t)(n_ex - 1) : -1;
        for (size_t d = n_ex - 1; d-- > 0;) {
            double t_now = grid[d + 1], t_next = grid[d + 2];
            double disc = std::exp(-mc.rate * (t_next - t_now));
            std::vector<double> xs, ys;
            for (size_t i = 0; i < np; ++i)
                if (payoff[d][i] > 0.0) { xs.push_back(spots[d][i]); ys.push_back(value[i] * disc); }
            bool have = xs.size() >= (size_t)n_basis;
            std::vector<double> coef;
            if (have) coef = basis == 1 ? laguerre_fit(xs, ys, (size_t)n_basis, m.s0) : poly_fit(xs, ys, (size_t)n_basis);
            for (size_t i = 0; i < np; ++i) {
                double discounted = value[i] * disc;
                if (payoff[d][i] > 0.0) {
                    double cont = !have ? discounted
                                  : basis == 1 ? laguerre_eval(coef, spots[d][i], m.s0) : poly_eval(coef, spots[d][i]);
                    value[i] = payoff[d][i] > cont ? payoff[d][i] : discounted;
                    if (payoff[d][i] > cont) exi[i] = (int32_t)d;
                    if (have) mrg[i] = std::min(mrg[i], std::fabs(payoff[d][i] - cont));
                } else {
                    value[i] = discounted;
                }
            }
        }
        double disc0 = std::exp(-mc.rate * grid[1]);
        for (auto &v : value) v *= disc0;
        *out = summarize(value);
        if (per_path) memcpy(per_path, value.data(), value.size() * sizeof(double));
        if (ex_index) memcpy(ex_index, exi.data(), exi.size() * sizeof(int32_t));
        if (margin) memcpy(margin, mrg.data(), mrg.size() * sizeof(double));
    });
}

int ko_price_american_basis(const char *json, const kx_model *model, const kx_mc_config *cfg, const double *dates,
                            size_t n_dates, int n_basis, int basis, kx_price_result *out, double *per_path) {
    return ko_price_american_detail(json, model, cfg, dates, n_dates, n_basis, basis, out, per_path, nullptr, nullptr);
}

int ko_price_american(const char *json, const kx_model *model, const kx_mc_config *cfg, const double *dates,
                      size_t n_dates, int n_basis, kx_price_result *out, double *per_path) {
    return ko_price_american_basis(json, model, cfg, dates, n_dates, n_basis, 0, out, per_path);
}

// present_value of a contract on one hand-built path (tests/observable.rs
// builds paths this way): times[n], spot values of `asset`, discount rate.
int ko_value_on_path(const char *json, const double *times, const double *values, size_t n, const char *asset,
                     double rate, double *out) {
    return run([&] {
        ConP c = parse_contract(json);
        std::vector<double> g(times, times + n);
        std::string a = asset ? asset : "ASSET";
        PathView pv{&g, values, &a};
        *out = present_value(*c, pv, g, rate);
    });
}

// ---- closed forms used as oracle values ------------------------------------
double ko_norm_cdf_as(double x) { return norm_cdf_as(x); }

// numerics.rs:63-71 (with the A&S cdf, as the reference)
double ko_bs_call(double s, double k, double t, double r, double sigma) {
    if (t <= 0.0 || sigma <= 0.0) return std::max(s - k * std::exp(-r * t), 0.0);
    double vst = sigma * std::sqrt(t);
    double d1 = (std::log(s / k) + (r + 0.5 * sigma * sigma) * t) / vst;
    double d2 = d1 - vst;
    return s * norm_cdf_as(d1) - k * std::exp(-r * t) * norm_cdf_as(d2);
}
// numerics.rs:83-91
double ko_bs_put(double s, double k, double t, double r, double sigma) {
    if (t <= 0.0 || sigma <= 0.0) return std::max(k * std::exp(-r * t) - s, 0.0);
    double vst = sigma * std::sqrt(t);
    double d1 = (std::log(s / k) + (r + 0.5 * sigma * sigma) * t) / vst;
    double d2 = d1 - vst;
    return k * std::exp(-r * t) * norm_cdf_as(-d2) - s * norm_cdf_as(-d1);
}
// Black-Scholes with the exact normal cdf (erfc) and its Greeks.
void ko_bs_call_greeks(double s, double k, double t, double r, double sigma, double *out5) {
    double vst = sigma * std::sqrt(t);
    double d1 = (std::log(s / k) + (r + 0.5 * sigma * sigma) * t) / vst;
    double d2 = d1 - vst;
    double pdf = std::exp(-0.5 * d1 * d1) / std::sqrt(2.0 * M_PI);
    out5[0] = s * norm_cdf_exact(d1) - k * std::exp(-r * t) * norm_cdf_exact(d2);
    out5[1] = norm_cdf_exact(d1);
    out5[2] = pdf / (s * vst);
    out5[3] = s * pdf * std::sqrt(t);
    out5[4] = k * t * std::exp(-r * t) * norm_cdf_exact(d2);
}

// Reiner-Rubinstein (1991) down-and-in call for H <= K, as in
// tests/barriers.rs:35-46; down-and-out = vanilla - down-and-in.
double ko_down_and_out_call(double s, double k, double h, double r, double sigma, double t) {
    double lambda = (r + 0.5 * sigma * sigma) / (sigma * sigma);
    double st = sigma * std::sqrt(t);
    double y = std::log(h * h / (s * k)) / st + lambda * st;
    double din = s * std::pow(h / s, 2.0 * lambda) * norm_cdf_as(y) -
                 k * std::exp(-r * t) * std::pow(h / s, 2.0 * lambda - 2.0) * norm_cdf_as(y - st);
    double d1 = (std::log(s / k) + (r + 0.5 * sigma * sigma) * t) / st;
    double van = s * norm_cdf_as(d1) - k * std::exp(-r * t) * norm_cdf_as(d1 - st);
    return van - din;
}

// Up-and-out call with barrier H > K, H > S, no rebate, continuous
// monitoring: the Reiner-Rubinstein (1991) formula as published in
// E.G. Haug, "The Complete Guide to Option Pricing Formulas" (2nd ed.,
// section 4.17.1): A - B + C - D with eta = -1, phi = 1, b = r (no carry
// adjustment). Discrete monitoring is handled by the caller with the
// Broadie-Glasserman-Kou shift H * exp(+0.5826 sigma sqrt(dt)).
double ko_up_and_out_call(double s, double k, double h, double r, double sigma, double t) {
    if (s >= h) return 0.0;
    double st = sigma * std::sqrt(t);
    double mu = (r - 0.5 * sigma * sigma) / (sigma * sigma);
    double x1 = std::log(s / k) / st + (1.0 + mu) * st;
    double x2 = std::log(s / h) / st + (1.0 + mu) * st;
    double y1 = std::log(h * h / (s * k)) / st + (1.0 + mu) * st;
    double y2 = std::log(h / s) / st + (1.0 + mu) * st;
    const double phi = 1.0, eta = -1.0;
    double df = std::exp(-r * t);
    auto N = norm_cdf_exact;
    double A = phi * s * N(phi * x1) - phi * k * df * N(phi * x1 - phi * st);
    double B = phi * s * N(phi * x2) - phi * k * df * N(phi * x2 - phi * st);
    double C = phi * s * std::pow(h / s, 2.0 * (mu + 1.0)) * N(eta * y1) -
               phi * k * df * std::pow(h / s, 2.0 * mu) * N(eta * y1 - eta * st);
    double D = phi * s * std::pow(h / s, 2.0 * (mu + 1.0)) * N(eta * y2) -
               phi * k * df * std::pow(h / s, 2.0 * mu) * N(eta * y2 - eta * st);
    return A - B + C - D;
}

// Heston (1993) European call by Fourier inversion, in the characteristic
// function form of Albrecher, Mayer, Schoutens and Tistaert, "The little
// Heston trap" (Wilmott, 2007), which stays on the principal branch of the
// complex logarithm: C = S0 P1 - K e^{-rT} P2 with
// Pj = 1/2 + (1/pi) int_0^inf Re[e^{-iu ln K} f_j(u) / (iu)] du,
// f_2(u) = phi(u), f_1(u) = phi(u - i) / phi(-i), phi the characteristic
// function of ln S_T. The integral runs over (0, 200] by composite Simpson
// with 20000 panels. Continuous-time model: the value the discretised
// schemes (simulator.rs:506-541, full truncation) converge to as dt -> 0.
// Not in the reference (it has no Heston closed form).
static std::complex<double> heston_cf(std::complex<double> u, double s0, double t, double r, double v0, double kappa,
                                      double theta, double sv, double rho) {
    using cd = std::complex<double>;
    const cd i(0.0, 1.0);
    const double sv2 = sv * sv;
    const cd b = kappa - rho * sv * i * u;
    const cd d = std::sqrt(b * b + sv2 * (i * u + u * u));
    const cd g = (b - d) / (b + d);
    const cd e = std::exp(-d * t);
    const cd A = i * u * (std::log(s0) + r * t);
    const cd B = kappa * theta / sv2 * ((b - d) * t - 2.0 * std::log((1.0 - g * e) / (1.0 - g)));
    const cd Cc = v0 / sv2 * (b - d) * (1.0 - e) / (1.0 - g * e);
    return std::exp(A + B + Cc);
}

double ko_heston_call(double s0, double k, double t, double r, double v0, double kappa, double theta, double sigma_v,
                      double rho) {
    using cd = std::complex<double>;
    const cd i(0.0, 1.0);
    const double lk = std::log(k);
    const cd phi_mi = heston_cf(cd(0.0, -1.0), s0, t, r, v0, kappa, theta, sigma_v, rho);
    auto integrand = [&](double u, int j) {
        const cd uc(u, 0.0);
        const cd f = j == 1 ? heston_cf(uc - i, s0, t, r, v0, kappa, theta, sigma_v, rho) / phi_mi
                            : heston_cf(uc, s0, t, r, v0, kappa, theta, sigma_v, rho);
        return std::real(std::exp(-i * uc * lk) * f / (i * uc));
    };
    const int n = 20000;  // even
    const double a = 1e-8, bnd = 200.0, h = (bnd - a) / n;
    double p[2];
    for (int j = 1; j <= 2; ++j) {
        double acc = integrand(a, j) + integrand(bnd, j);
        for (int q = 1; q < n; ++q) acc += (q % 2 ? 4.0 : 2.0) * integrand(a + q * h, j);
        p[j - 1] = 0.5 + acc * h / 3.0 / M_PI;
    }
    return s0 * p[0] - k * std::exp(-r * t) * p[1];
}

// Cox-Ross-Rubinstein binomial tree for American options (tests/j17_lsm.rs:40-72).
double ko_crr_american(double s0, double k, double t, double r, double sigma, int n, int is_call) {
    double dt = t / n;
    double u = std::exp(sigma * std::sqrt(dt));
    double d = 1.0 / u;
    double disc = std::exp(-r * dt);
    double p = (std::exp(r * dt) - d) / (u - d);
    auto pay = [&](double s) { return is_call ? std::max(s - k, 0.0) : std::max(k - s, 0.0); };
    std::vector<double> v(n + 1);
    for (int j = 0; j <= n; ++j) v[j] = pay(s0 * std::pow(u, j) * std::pow(d, n - j));
    for (int step = n - 1; step >= 0; --step)
        for (int j = 0; j <= step; ++j) {
            double s = s0 * std::pow(u, j) * std::pow(d, step - j);
            double cont = disc * (p * v[j + 1] + (1.0 - p) * v[j]);
            v[j] = std::max(cont, pay(s));
        }
    return v[0];
}

}  // extern "C"
