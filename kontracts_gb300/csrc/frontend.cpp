// frontend.cpp — contract JSON -> AST -> Plan/grid -> lowered KxProgram.
#include "frontend.hpp"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>

namespace kx {

void raise(kx_status code, const std::string &msg) { throw Error{code, msg}; }
// the reference's messages (src/error.rs:11-15), with the payload kept apart
void raise_time_out_of_range(double t) {
    Error e{KX_TIME_OUT_OF_RANGE, "date d'observation hors de la timeline : " + std::to_string(t)};
    e.time = t;
    throw e;
}
void raise_step_out_of_range(uint64_t step) {
    Error e{KX_STEP_OUT_OF_RANGE, "pas de temps hors de la trajectoire : index " + std::to_string(step)};
    e.step = step;
    throw e;
}

// ============================================================================
// serde_json reader for the externally tagged enums of src/ast.rs.
// `Contract::from_json` (ast.rs:215) accepts exactly this shape:
//   unit variant      "Zero"
//   newtype variant   {"One":"USD"}, {"Give":C}, {"Const":1.0}, {"Not":Cond}
//   tuple variant     {"And":[C,C]}, {"Scale":[Obs,C]}, {"When":[Cond,C]}
//   struct variant    {"Average":{"obs":O,"from_year":x|null,"to_year":y|null}}
// ============================================================================
namespace {

struct Reader {
    const char *p, *e;

    [[noreturn]] void bad(const std::string &what) {
        raise(KX_SERDE, what + " at offset " + std::to_string(p - start));
    }
    const char *start;

    void ws() {
        while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool peek(char c) {
        ws();
        return p < e && *p == c;
    }
    void expect(char c) {
        ws();
        if (p >= e || *p != c) bad(std::string("expected '") + c + "'");
        ++p;
    }
    bool literal(const char *lit) {
        ws();
        size_t n = strlen(lit);
        if ((size_t)(e - p) >= n && !memcmp(p, lit, n)) { p += n; return true; }
        return false;
    }
    std::string str() {
        expect('"');
        std::string s;
        while (true) {
            if (p >= e) bad("unterminated string");
            char c = *p++;
            if (c == '"') break;
            if (c != '\\') { s.push_back(c); continue; }
            if (p >= e) bad("bad escape");
            char x = *p++;
            switch (x) {
            case '"': case '\\': case '/': s.push_back(x); break;
            case 'b': s.push_back('\b'); break;
            case 'f': s.push_back('\f'); break;
            case 'n': s.push_back('\n'); break;
            case 'r': s.push_back('\r'); break;
            case 't': s.push_back('\t'); break;
            case 'u': {
                if (e - p < 4) bad("short \\u escape");
                char hex[5] = {p[0], p[1], p[2], p[3], 0};
                p += 4;
                unsigned cp = (unsigned)strtoul(hex, nullptr, 16);
                if (cp < 0x80) {
                    s.push_back((char)cp);
                } else if (cp < 0x800) {
                    s.push_back((char)(0xC0 | (cp >> 6)));
                    s.push_back((char)(0x80 | (cp & 0x3F)));
                } else {
                    s.push_back((char)(0xE0 | (cp >> 12)));
                    s.push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
                    s.push_back((char)(0x80 | (cp & 0x3F)));
                }
                break;
            }
            default: bad("bad escape");
            }
        }
        return s;
    }
    double number() {
        ws();
        const char *s0 = p;
        if (p < e && *p == '-') ++p;
        if (p >= e || !(*p >= '0' && *p <= '9')) bad("expected a number");
        while (p < e && ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' || *p == 'E' || *p == '+' || *p == '-'))
            ++p;
        std::string tok(s0, p);
        char *end = nullptr;
        double v = strtod(tok.c_str(), &end);
        if (!end || *end) bad("malformed number");
        if (!std::isfinite(v)) bad("number out of range");
        return v;
    }
    // {"Tag": ...} or "Tag"; returns the tag, leaves the payload (if any) next.
    std::string tag(bool &unit) {
        ws();
        if (peek('"')) { unit = true; return str(); }
        expect('{');
        unit = false;
        std::string t = str();
        expect(':');
        return t;
    }
    void close(bool unit) {
        if (!unit) expect('}');
    }
};

NodeP mk(NK k) {
    auto n = std::make_unique<Node>();
    n->k = k;
    return n;
}

NodeP read_obs(Reader &r);
NodeP read_cond(Reader &r);
NodeP read_contract(Reader &r);

void need_payload(Reader &r, bool unit, const std::string &t) {
    if (unit) r.bad("variant `" + t + "` expects a payload");
}

NodeP read_obs(Reader &r) {
    bool unit;
    std::string t = r.tag(unit);
    static const std::map<std::string, NK> bin = {{"Add", NK::Add}, {"Sub", NK::Sub}, {"Mul", NK::Mul},
                                                  {"Div", NK::Div}, {"Max", NK::Max}, {"Min", NK::Min}};
    NodeP n;
    need_payload(r, unit, t);
    if (t == "Const") {
        n = mk(NK::Const);
        n->num = r.number();
    } else if (t == "Spot") {
        n = mk(NK::Spot);
        n->text = r.str();
    } else if (t == "Neg" || t == "RunningMax" || t == "RunningMin") {
        n = mk(t == "Neg" ? NK::Neg : t == "RunningMax" ? NK::RunningMax : NK::RunningMin);
        n->kid.push_back(read_obs(r));
    } else if (bin.count(t)) {
        n = mk(bin.at(t));
        r.expect('[');
        n->kid.push_back(read_obs(r));
        r.expect(',');
        n->kid.push_back(read_obs(r));
        r.expect(']');
    } else if (t == "Average") {
        n = mk(NK::Average);
        auto opt = [&](bool &has, double &v) {
            if (r.literal("null")) { has = false; return; }
            has = true;
            v = r.number();
        };
        if (r.peek('[')) {  // serde also accepts a struct variant as a sequence
            r.expect('[');
            n->kid.push_back(read_obs(r));
            r.expect(',');
            opt(n->has_from, n->from);
            r.expect(',');
            opt(n->has_to, n->to);
            r.expect(']');
        } else {
            r.expect('{');
            bool first = true, got_obs = false;
            while (!r.peek('}')) {
                if (!first) r.expect(',');
                first = false;
                std::string f = r.str();
                r.expect(':');
                if (f == "obs") { n->kid.push_back(read_obs(r)); got_obs = true; }
                else if (f == "from_year") opt(n->has_from, n->from);
                else if (f == "to_year") opt(n->has_to, n->to);
                else r.bad("unknown field `" + f + "` in Average");
            }
            r.expect('}');
            if (!got_obs) r.bad("missing field `obs`");
        }
    } else {
        r.bad("unknown variant `" + t + "` of Observable");
    }
    r.close(unit);
    return n;
}

NodeP read_cond(Reader &r) {
    bool unit;
    std::string t = r.tag(unit);
    need_payload(r, unit, t);
    static const std::map<std::string, NK> cmp = {{"Ge", NK::Ge}, {"Gt", NK::Gt}, {"Le", NK::Le}, {"Lt", NK::Lt}};
    NodeP n;
    if (t == "Bool") {
        n = mk(NK::Bool);
        if (r.literal("true")) n->flag = true;
        else if (r.literal("false")) n->flag = false;
        else r.bad("Bool expects a boolean");
    } else if (t == "At") {
        n = mk(NK::At);
        n->num = r.number();
    } else if (cmp.count(t)) {
        n = mk(cmp.at(t));
        r.expect('[');
        n->kid.push_back(read_obs(r));
        r.expect(',');
        n->kid.push_back(read_obs(r));
        r.expect(']');
    } else if (t == "And" || t == "Or") {
        n = mk(t == "And" ? NK::And : NK::Or);
        r.expect('[');
        n->kid.push_back(read_cond(r));
        r.expect(',');
        n->kid.push_back(read_cond(r));
        r.expect(']');
    } else if (t == "Not") {
        n = mk(NK::Not);
        n->kid.push_back(read_cond(r));
    } else {
        r.bad("unknown variant `" + t + "` of Condition");
    }
    r.close(unit);
    return n;
}

NodeP read_contract(Reader &r) {
    bool unit;
    std::string t = r.tag(unit);
    NodeP n;
    if (t == "Zero") {
        n = mk(NK::Zero);
        if (!unit && !r.literal("null")) r.bad("Zero takes no payload");
    } else {
        need_payload(r, unit, t);
        if (t == "One") {
            n = mk(NK::One);
            n->text = r.str();
        } else if (t == "Give") {
            n = mk(NK::Give);
            n->kid.push_back(read_contract(r));
        } else if (t == "And" || t == "Or") {
            n = mk(t == "And" ? NK::CAnd : NK::COr);
            r.expect('[');
            n->kid.push_back(read_contract(r));
            r.expect(',');
            n->kid.push_back(read_contract(r));
            r.expect(']');
        } else if (t == "Scale") {
            n = mk(NK::Scale);
            r.expect('[');
            n->kid.push_back(read_obs(r));
            r.expect(',');
            n->kid.push_back(read_contract(r));
            r.expect(']');
        } else if (t == "When" || t == "Anytime" || t == "Until") {
            n = mk(t == "When" ? NK::When : t == "Anytime" ? NK::Anytime : NK::Until);
            r.expect('[');
            n->kid.push_back(read_cond(r));
            r.expect(',');
            n->kid.push_back(read_contract(r));
            r.expect(']');
        } else {
            r.bad("unknown variant `" + t + "` of Contract");
        }
    }
    r.close(unit);
    return n;
}

}  // namespace

NodeP parse_contract_json(const char *json) {
    if (!json) raise(KX_INVALID_ARGUMENT, "contract json is NULL");
    Reader r{json, json + strlen(json), json};
    NodeP n = read_contract(r);
    r.ws();
    if (r.p != r.e) r.bad("trailing characters");
    return n;
}

// ============================================================================
// Compiler — restates src/compiler.rs:54-189.
// ============================================================================
std::vector<double> sort_dedup(std::vector<double> v) {  // compiler.rs:185-189
    std::sort(v.begin(), v.end());
    size_t w = 0;
    for (size_t i = 0; i < v.size(); ++i)
        if (w == 0 || !(std::fabs(v[i] - v[w - 1]) < 1e-12)) v[w++] = v[i];
    v.resize(w);
    return v;
}

namespace {
struct Walk {
    std::set<std::string> assets;
    std::vector<double> dates;
    bool fine = false;
};

bool is_price_dependent(const Node &c) {  // compiler.rs:173-182
    switch (c.k) {
    case NK::Ge: case NK::Gt: case NK::Le: case NK::Lt: return true;
    case NK::And: case NK::Or: return is_price_dependent(*c.kid[0]) || is_price_dependent(*c.kid[1]);
    case NK::Not: return is_price_dependent(*c.kid[0]);
    default: return false;
    }
}

void walk(const Node &n, Walk &w) {
    switch (n.k) {
    case NK::Spot: w.assets.insert(n.text); return;
    case NK::Average: case NK::RunningMax: case NK::RunningMin:  // compiler.rs:139-145
        w.fine = true;
        break;
    case NK::At:  // compiler.rs:151-160
        if (!std::isfinite(n.num) || n.num < 0.0)
            raise(KX_MALFORMED_CONTRACT, "invalid acquisition date: " + std::to_string(n.num));
        w.dates.push_back(n.num);
        return;
    case NK::When: case NK::Anytime: case NK::Until:  // compiler.rs:111-119
        walk(*n.kid[0], w);
        if (is_price_dependent(*n.kid[0])) w.fine = true;
        walk(*n.kid[1], w);
        return;
    default: break;
    }
    for (auto &k : n.kid) walk(*k, w);
}
}  // namespace

Plan compile_plan(const Node &contract) {  // compiler.rs:69-86
    Walk w;
    walk(contract, w);
    Plan p;
    for (double d : w.dates) if (d > p.horizon) p.horizon = d;
    p.assets.assign(w.assets.begin(), w.assets.end());
    p.fixed_dates = sort_dedup(w.dates);
    p.needs_fine_grid = w.fine;
    return p;
}

std::vector<double> time_grid_forced(const Plan &p, uint32_t spy, bool force) {  // compiler.rs:54-65
    std::vector<double> pts;
    pts.reserve(p.fixed_dates.size() + 2);
    pts.push_back(0.0);
    for (double d : p.fixed_dates) pts.push_back(d);
    pts.push_back(p.horizon);
    if ((p.needs_fine_grid || force) && p.horizon > 0.0 && spy > 0) {
        double nd = std::ceil(p.horizon * (double)spy);
        if (nd > 5e7) raise(KX_INVALID_ARGUMENT, "time grid too large");
        size_t n = (size_t)nd;
        for (size_t k = 1; k <= n; ++k) pts.push_back(p.horizon * (double)k / (double)n);
    }
    return sort_dedup(std::move(pts));
}

// ============================================================================
// Lowering
// ============================================================================
namespace {

struct Lowerer {
    Lowered &L;
    KxProgram &P;
    std::vector<std::pair<const Node *, int>> acc_nodes;  // dedup by structure
    explicit Lowerer(Lowered &l) : L(l), P(l.prog) {}

    void emit(uint8_t op, uint16_t arg = 0) {
        if (P.n_code >= KX_MAX_CODE) raise(KX_UNSUPPORTED, "contract too large for the device program table");
        P.code[P.n_code++] = KxIns{op, 0, arg};
    }
    uint16_t konst(double c) {
        for (int i = 0; i < P.n_const; ++i)
            if (memcmp(&P.cpool[i], &c, sizeof c) == 0) return (uint16_t)i;
        if (P.n_const >= KX_MAX_CONST) raise(KX_UNSUPPORTED, "too many constants in contract");
        P.cpool[P.n_const] = c;
        return (uint16_t)P.n_const++;
    }
    static bool same(const Node &a, const Node &b) {
        if (a.k != b.k || a.num != b.num || a.flag != b.flag || a.text != b.text || a.has_from != b.has_from ||
            a.has_to != b.has_to || (a.has_from && a.from != b.from) || (a.has_to && a.to != b.to) ||
            a.kid.size() != b.kid.size())
            return false;
        for (size_t i = 0; i < a.kid.size(); ++i)
            if (!same(*a.kid[i], *b.kid[i])) return false;
        return true;
    }

    // Accumulator for Average / RunningMax / RunningMin; inner accumulators
    // are created first so their slots precede (update order = slot order).
    int accumulator(const Node &n) {
        for (auto &an : acc_nodes)
            if (same(*an.first, n)) return an.second;
        const Node &inner = *n.kid[0];
        KxAcc a{};
        a.kind = n.k == NK::RunningMax ? ACC_MAX : n.k == NK::RunningMin ? ACC_MIN : ACC_SUM;
        if (inner.k == NK::Spot) {
            a.inner = IK_SPOT;
            a.pad = (uint8_t)note_spot(inner);  // the asset it reads
        } else {
            a.inner = IK_GENERAL;
            int start = P.n_code;
            int d = obs(inner);
            if (d > P.max_stack) P.max_stack = d;
            a.code_off = (uint16_t)start;
            a.code_len = (uint16_t)(P.n_code - start);
        }
        if (P.n_acc >= KX_MAX_ACC) raise(KX_UNSUPPORTED, "too many running/average observables (max 8)");
        int slot = P.n_acc++;
        a.fixed = n.k == NK::Average && n.has_to;
        P.acc[slot] = a;
        AccWindow w;
        if (n.k == NK::Average) {
            w.has_from = n.has_from; w.from = n.from;
            w.has_to = n.has_to; w.to = n.to;
            if (!n.has_to) L.has_running_average = true;
            P.err_capable = 1;
        }
        L.acc_window.push_back(w);
        P.spot_each_step = 1;
        acc_nodes.emplace_back(&n, slot);
        return slot;
    }
    // Index of the spot's asset in the program's asset list (order of appearance).
    int note_spot(const Node &n) {
        auto it = std::find(L.spot_assets.begin(), L.spot_assets.end(), n.text);
        if (it != L.spot_assets.end()) return (int)(it - L.spot_assets.begin());
        L.spot_assets.push_back(n.text);
        return (int)L.spot_assets.size() - 1;
    }

    // Observable -> postfix code; returns the stack depth it needs.
    int obs(const Node &n) {
        switch (n.k) {
        case NK::Const: emit(OP_CONST, konst(n.num)); return 1;
        case NK::Spot: emit(OP_SPOT, (uint16_t)note_spot(n)); return 1;
        case NK::Neg: { int d = obs(*n.kid[0]); emit(OP_NEG); return d; }
        case NK::Add: case NK::Sub: case NK::Mul: case NK::Div: case NK::Max: case NK::Min: {
            int a = obs(*n.kid[0]);
            int b = obs(*n.kid[1]);
            static const std::map<NK, uint8_t> ops = {{NK::Add, OP_ADD}, {NK::Sub, OP_SUB}, {NK::Mul, OP_MUL},
                                                      {NK::Div, OP_DIV}, {NK::Max, OP_MAX}, {NK::Min, OP_MIN}};
            emit(ops.at(n.k));
            return std::max(a, b + 1);
        }
        case NK::Average: case NK::RunningMax: case NK::RunningMin: {
            // note: the slot's inner code is emitted by accumulator(); its code
            // lives in the same table but is only run by the accumulator update.
            int start_code = P.n_code;
            (void)start_code;
            int slot = accumulator(n);
            emit(OP_ACC, (uint16_t)slot);
            return 1;
        }
        default: raise(KX_MALFORMED_CONTRACT, "not an observable");
        }
    }

    int cond(const Node &n) {
        switch (n.k) {
        case NK::Bool: emit(n.flag ? OP_TRUE : OP_FALSE); return 1;
        case NK::At: {
            if ((int)L.at_dates.size() >= KX_MAX_AT) raise(KX_UNSUPPORTED, "too many date conditions");
            L.at_dates.push_back(n.num);
            emit(OP_AT, (uint16_t)(L.at_dates.size() - 1));
            return 1;
        }
        case NK::Ge: case NK::Gt: case NK::Le: case NK::Lt: {
            int a = obs(*n.kid[0]);
            int b = obs(*n.kid[1]);
            static const std::map<NK, uint8_t> ops = {{NK::Ge, OP_GE}, {NK::Gt, OP_GT}, {NK::Le, OP_LE}, {NK::Lt, OP_LT}};
            emit(ops.at(n.k));
            return std::max(a, b + 1);
        }
        case NK::And: case NK::Or: {
            int a = cond(*n.kid[0]);
            int b = cond(*n.kid[1]);
            emit(n.k == NK::And ? OP_AND : OP_OR);
            return std::max(a, b + 1);
        }
        case NK::Not: { int d = cond(*n.kid[0]); emit(OP_NOT); return d; }
        default: raise(KX_MALFORMED_CONTRACT, "not a condition");
        }
    }

    // Code that the program itself must never run inline (accumulator inner
    // code is emitted while an enclosing expression is being emitted), so each
    // expression is compiled into a scratch buffer first and then appended.
    struct Code {
        int off, len, depth;
    };
    template <class F>
    Code compile_expr(F &&f) {
        // Inner accumulator programs are appended to the table as they are
        // created; to keep the outer program contiguous it is compiled twice:
        // first to create every accumulator (discarded), then for real.
        int save = P.n_code;
        f();
        P.n_code = save;  // accumulators now exist; their code sits before `save`? no: see below
        int start = P.n_code;
        int d = f();
        return Code{start, P.n_code - start, d};
    }

    int trig_count = 0, leaf_count = 0;

    int new_trig(uint8_t kind, const Node &c, uint32_t arm_by_when, int acquiring) {
        if (P.n_trig >= KX_MAX_TRIG) raise(KX_UNSUPPORTED, "too many when/anytime/until nodes (max 32)");
        int i = P.n_trig++;
        KxTrig &t = P.trig[i];
        t = KxTrig{};
        t.kind = kind;
        (void)arm_by_when;
        if (acquiring < 0) P.root_arm |= 1u << i;
        else P.trig[acquiring].fire_arm |= 1u << i;
        if (kind == TK_WHEN) P.when_mask |= 1u << i;
        else P.until_mask |= 1u << i;
        if (!is_price_dependent(c)) {
            t.cond_kind = CK_TIME;
            P.time_mask |= 1u << i;
            if ((int)L.time_cond.size() <= i) L.time_cond.resize(i + 1, nullptr);
            L.time_cond[i] = &c;
            // At dates inside time conditions are still validated by the compiler walk.
        } else {
            P.price_mask |= 1u << i;
            Code code = compile_cond(c);
            t.code_off = (uint16_t)code.off;
            t.code_len = (uint16_t)code.len;
            if (code.depth > P.max_stack) P.max_stack = code.depth;
            const Node *lhs = c.kid.size() == 2 ? c.kid[0].get() : nullptr;
            const Node *rhs = c.kid.size() == 2 ? c.kid[1].get() : nullptr;
            bool is_cmp = c.k == NK::Ge || c.k == NK::Gt || c.k == NK::Le || c.k == NK::Lt;
            uint8_t cmp = c.k == NK::Ge ? CMP_GE : c.k == NK::Gt ? CMP_GT : c.k == NK::Le ? CMP_LE : CMP_LT;
            if (is_cmp && lhs->k == NK::Spot && rhs->k == NK::Const && rhs->num > 0.0) {
                t.cond_kind = CK_SPOT_CMP;
                t.cmp = cmp;
                t.spot_slot = (uint8_t)L.spot_cmp.size();
                L.spot_cmp.push_back(SpotCmp{rhs->num});
            } else if (is_cmp && lhs->k == NK::Const && rhs->k == NK::Spot && lhs->num > 0.0) {
                // c >= S  <=>  S <= c, etc.
                static const uint8_t flip[4] = {CMP_LE, CMP_LT, CMP_GE, CMP_GT};
                t.cond_kind = CK_SPOT_CMP;
                t.cmp = flip[cmp];
                t.spot_slot = (uint8_t)L.spot_cmp.size();
                L.spot_cmp.push_back(SpotCmp{lhs->num});
            } else {
                t.cond_kind = CK_GENERAL;
                P.spot_each_step = 1;
            }
        }
        return i;
    }

    Code compile_cond(const Node &c) {
        // Create accumulators first (they append their own inner code), then
        // emit the condition program contiguously.
        prepass(c);
        int start = P.n_code;
        int d = cond(c);
        return Code{start, P.n_code - start, d};
    }
    Code compile_obs(const Node &o) {
        prepass(o);
        int start = P.n_code;
        int d = obs(o);
        return Code{start, P.n_code - start, d};
    }
    // Instantiate every accumulator below `n` (post-order: inner ones first).
    void prepass(const Node &n) {
        for (auto &k : n.kid) prepass(*k);
        if (n.k == NK::Average || n.k == NK::RunningMax || n.k == NK::RunningMin) {
            bool exists = false;
            for (auto &an : acc_nodes) if (same(*an.first, n)) exists = true;
            if (!exists) accumulator(n);
        }
    }

    // Contract walk. `acq` = acquiring when-slot (-1: acquired at step 0),
    // `untils` = until-slots above, `sign`, `scales` = enclosing observables.
    void contract(const Node &n, int acq, uint32_t untils, double sign, std::vector<const Node *> &scales) {
        switch (n.k) {
        case NK::Zero: return;
        case NK::One: leaf(acq, untils, sign, scales); return;
        case NK::Give: contract(*n.kid[0], acq, untils, -sign, scales); return;
        case NK::CAnd:
            contract(*n.kid[0], acq, untils, sign, scales);
            contract(*n.kid[1], acq, untils, sign, scales);
            return;
        case NK::COr: raise(KX_UNSUPPORTED, "or (optimal choice needs LSM)");  // pricer.rs:416
        case NK::Scale:
            scales.push_back(n.kid[0].get());
            contract(*n.kid[1], acq, untils, sign, scales);
            scales.pop_back();
            return;
        case NK::When: case NK::Anytime: {
            int i = new_trig(TK_WHEN, *n.kid[0], 0, acq);
            contract(*n.kid[1], i, untils, sign, scales);
            return;
        }
        case NK::Until: {
            int i = new_trig(TK_UNTIL, *n.kid[0], 0, acq);
            contract(*n.kid[1], acq, untils | (1u << i), sign, scales);
            return;
        }
        default: raise(KX_MALFORMED_CONTRACT, "not a contract");
        }
    }

    void leaf(int acq, uint32_t untils, double sign, const std::vector<const Node *> &scales) {
        if (P.n_leaf >= KX_MAX_LEAF) raise(KX_UNSUPPORTED, "too many one(...) leaves (max 32)");
        int j = P.n_leaf++;
        KxLeaf &l = P.leaf[j];
        l = KxLeaf{};
        l.sign = sign;
        P.all_leaves |= 1u << j;
        if (acq < 0) P.root_leaves |= 1u << j;
        else P.trig[acq].leaves |= 1u << j;
        for (int u = 0; u < KX_MAX_TRIG; ++u)
            if (untils >> u & 1u) P.trig[u].leaves |= 1u << j;
        if (scales.empty()) {
            l.kind = AK_CONST;
            P.simple_leaves |= 1u << j;
            return;
        }
        // amount = scale_1 * scale_2 * ... (then * sign); pricer.rs:391-395
        // multiplies the flow amount by each observable from the innermost out.
        for (auto *s : scales) prepass(*s);
        int start = P.n_code;
        int depth = 0;
        // innermost scale first, as cashflows() applies them on the way up
        // from the leaf: amt = ((1 * s_inner) * ...) * s_outer.
        bool first = true;
        for (auto it = scales.rbegin(); it != scales.rend(); ++it) {
            int d = obs(**it);
            depth = std::max(depth, first ? d : d + 1);
            if (!first) emit(OP_MUL);
            first = false;
        }
        if (sign < 0) emit(OP_NEG);
        l.kind = AK_GENERAL;
        l.code_off = (uint16_t)start;
        l.code_len = (uint16_t)(P.n_code - start);
        if (depth > P.max_stack) P.max_stack = depth;
        fast_form(l);
    }

    // Recognise the amounts that have a closed form (KxFastAmount).
    void fast_form(KxLeaf &l) {
        const KxIns *c = P.code + l.code_off;
        int n = l.code_len;
        if (n >= 1 && c[n - 1].op == OP_NEG) --n;  // the sign is kept in l.sign
        const int j = (int)(&l - P.leaf);
        auto is_zero = [&](const KxIns &i) { return i.op == OP_CONST && P.cpool[i.arg] == 0.0; };
        if (n == 1 && c[0].op == OP_SPOT) {
            l.fast = FA_SPOT;
        } else if (n == 1 && c[0].op == OP_CONST) {
            l.fast = FA_CONST;
            l.fast_k = (uint8_t)c[0].arg;
        } else if (n == 5 && c[2].op == OP_SUB && is_zero(c[3]) && c[4].op == OP_MAX) {
            if (c[0].op == OP_SPOT && c[1].op == OP_CONST) {
                l.fast = FA_CALL;
                l.fast_k = (uint8_t)c[1].arg;
            } else if (c[0].op == OP_CONST && c[1].op == OP_SPOT) {
                l.fast = FA_PUT;
                l.fast_k = (uint8_t)c[0].arg;
            }
        }
        if (l.fast != FA_NONE && !l.err_capable) P.simple_leaves |= 1u << j;
    }
};

bool subtree_has(const Node &n, NK k) {
    if (n.k == k) return true;
    for (auto &c : n.kid) if (subtree_has(*c, k)) return true;
    return false;
}

}  // namespace

void lower(Program &p) {
    Lowered &L = p.low;
    L = Lowered{};
    memset(&L.prog, 0, sizeof(KxProgram));
    Lowerer lw(L);
    std::vector<const Node *> scales;
    lw.contract(*p.ast, -1, 0u, 1.0, scales);
    if (L.prog.max_stack > KX_MAX_STACK) raise(KX_UNSUPPORTED, "observable expression too deep for the device stack");
    L.prog.n_spot_cmp = (int32_t)L.spot_cmp.size();
    L.prog.n_at = (int32_t)L.at_dates.size();
    L.time_cond.resize(L.prog.n_trig, nullptr);
    // Leaves whose amount reads an average can raise MalformedContract.
    for (int j = 0; j < L.prog.n_leaf; ++j) {
        const KxLeaf &l = L.prog.leaf[j];
        for (int c = l.code_off; c < l.code_off + l.code_len; ++c)
            if (L.prog.code[c].op == OP_ACC && L.prog.acc[L.prog.code[c].arg].kind == ACC_SUM)
                L.prog.leaf[j].err_capable = 1;
    }
    (void)subtree_has;
}

// ============================================================================
// Models and binding
// ============================================================================
Model model_from_c(const kx_model *m) {
    if (!m) raise(KX_INVALID_ARGUMENT, "model is NULL");
    Model o;
    o.kind = m->kind;
    o.scheme = m->heston_scheme;
    o.s0 = m->s0; o.mu = m->mu; o.sigma = m->sigma;
    o.v0 = m->v0; o.kappa = m->kappa; o.theta = m->theta; o.sigma_v = m->sigma_v; o.rho = m->rho; o.r = m->r;
    o.asset = m->asset ? m->asset : "ASSET";
    if (o.kind != KX_MODEL_GBM && o.kind != KX_MODEL_HESTON) raise(KX_INVALID_ARGUMENT, "unknown model kind");
    if (o.kind == KX_MODEL_HESTON && o.scheme != KX_HESTON_REFERENCE_FLOOR && o.scheme != KX_HESTON_FULL_TRUNCATION)
        raise(KX_INVALID_ARGUMENT, "unknown Heston scheme");
    return o;
}

void validate_model(const Model &m) {
    if (m.kind == KX_MODEL_MULTI_GBM) {
        for (double sg : m.a_sigma)
            if (sg < 0.0) raise(KX_MALFORMED_CONTRACT, "CorrelatedGbmN: every volatility must be >= 0");
    } else if (m.kind == KX_MODEL_GBM) {
        if (m.sigma < 0.0) raise(KX_MALFORMED_CONTRACT, "GBM sigma must be non-negative");  // simulator.rs:221-225
    } else {                                                                               // simulator.rs:556-580
        if (!(m.rho >= -1.0 && m.rho <= 1.0)) raise(KX_MALFORMED_CONTRACT, "Heston rho must be in [-1, 1]");
        if (m.v0 < 0.0) raise(KX_MALFORMED_CONTRACT, "Heston v0 must be non-negative");
        if (m.sigma_v < 0.0) raise(KX_MALFORMED_CONTRACT, "Heston sigma_v must be non-negative");
        if (m.theta < 0.0) raise(KX_MALFORMED_CONTRACT, "Heston theta must be non-negative");
        if (m.kappa < 0.0) raise(KX_MALFORMED_CONTRACT, "Heston kappa must be non-negative");
    }
}

void validate_grid(const std::vector<double> &g) {  // simulator.rs:413-428
    if (g.empty()) raise(KX_INCONSISTENT_PATH, "empty grid");
    double prev = 0.0;
    for (double t : g) {
        if (t < prev) raise(KX_INCONSISTENT_PATH, "grid not increasing near " + std::to_string(t));
        prev = t;
    }
    // Engine requirement: the path starts at t = 0 and every later point
    // advances (the reference skips zero steps; grids built by the compiler
    // or by the LSM driver never contain one).
    if (g[0] != 0.0) raise(KX_UNSUPPORTED, "grid must start at t = 0");
    for (size_t k = 1; k < g.size(); ++k)
        if (!(g[k] - g[k - 1] > 0.0)) raise(KX_UNSUPPORTED, "grid with a zero-length step");
}

namespace {
bool eval_time_cond(const Node &c, double t_now, const Lowered &) {
    switch (c.k) {
    case NK::Bool: return c.flag;
    case NK::At: return t_now + 1e-12 >= c.num;  // observable.rs:153-159
    case NK::And: return eval_time_cond(*c.kid[0], t_now, {}) && eval_time_cond(*c.kid[1], t_now, {});
    case NK::Or: return eval_time_cond(*c.kid[0], t_now, {}) || eval_time_cond(*c.kid[1], t_now, {});
    case NK::Not: return !eval_time_cond(*c.kid[0], t_now, {});
    default: raise(KX_MALFORMED_CONTRACT, "price-dependent node in a time condition");
    }
}
}  // namespace

void bind(const Lowered &low, const std::vector<double> &grid, const Model &m, double rate, KxProgram &P,
          StepTables &tab) {
    P = low.prog;
    const int n = (int)grid.size();
    P.n_times = n;
    if (m.kind == KX_MODEL_MULTI_GBM) {
        // the program's assets -> the model's factors (observable.rs:78-87): OP_SPOT and
        // spot accumulators read the factor's index; every price condition and amount goes
        // through the interpreter (the closed forms read one spot)
        std::vector<int> idx;
        for (auto &a : low.spot_assets) {
            auto it = std::find(m.assets.begin(), m.assets.end(), a);
            if (it == m.assets.end()) raise(KX_UNKNOWN_ASSET, a);
            idx.push_back((int)(it - m.assets.begin()));
        }
        for (int c = 0; c < P.n_code; ++c)
            if (P.code[c].op == OP_SPOT) P.code[c].arg = (uint16_t)idx[P.code[c].arg];
        for (int a = 0; a < P.n_acc; ++a)
            if (P.acc[a].inner == IK_SPOT) P.acc[a].pad = (uint8_t)idx[P.acc[a].pad];
        for (int i = 0; i < P.n_leaf; ++i) P.leaf[i].fast = FA_NONE;
        P.simple_leaves = 0;
        for (int i = 0; i < P.n_trig; ++i)
            if (P.trig[i].cond_kind == CK_SPOT_CMP) P.trig[i].cond_kind = CK_GENERAL;
        P.spot_each_step = 1;
    } else {
        for (auto &a : low.spot_assets)
            if (a != m.asset) raise(KX_UNKNOWN_ASSET, a);  // observable.rs:78-87
    }
    if (low.has_running_average)
        for (int e = 0; e + 1 < n; ++e)
            if (grid[e + 1] <= grid[e] + 1e-12)
                raise(KX_UNSUPPORTED, "grid points closer than 1e-12 under a running average");
    // OP_AT slots: first step with t + 1e-12 >= date.
    for (size_t s = 0; s < low.at_dates.size(); ++s) {
        int k = 0;
        while (k < n && !(grid[k] + 1e-12 >= low.at_dates[s])) ++k;
        P.at_index[s] = k;
    }
    // CK_SPOT_CMP thresholds: S cmp c  <=>  log(S/s0) cmp log(c/s0) (s0 > 0).
    for (int i = 0; i < P.n_trig; ++i) {
        KxTrig &t = P.trig[i];
        if (t.cond_kind == CK_SPOT_CMP) {
            if (m.s0 > 0.0) P.spot_thr[i] = std::log(low.spot_cmp[t.spot_slot].c / m.s0);
            else { t.cond_kind = CK_GENERAL; P.spot_each_step = 1; }
        }
    }
    // accumulator windows (observable.rs:103-134)
    for (int a = 0; a < P.n_acc; ++a) {
        KxAcc &A = P.acc[a];
        A.i_from = 0;
        A.i_to = INT32_MAX;
        A.e_min = 0;
        A.static_err = 0;
        A.inv_count = 0.0;
        if (A.kind != ACC_SUM) continue;
        const AccWindow &w = low.acc_window[a];
        double from = w.has_from ? w.from : 0.0;
        int i_from = 0;
        while (i_from < n && !(grid[i_from] >= from - 1e-12)) ++i_from;
        A.i_from = i_from;
        if (w.has_to) {
            int i_to = n - 1;
            while (i_to >= 0 && !(grid[i_to] <= w.to + 1e-12)) --i_to;
            A.i_to = i_to;
            int cnt = i_to - i_from + 1;
            if (from > w.to + 1e-12 || cnt <= 0) A.static_err = 1;
            A.inv_count = cnt > 0 ? (double)cnt : 0.0;  // window size (division, as the reference)
            A.e_min = i_to;                             // read before that = look-ahead
        } else {
            int e = 0;
            while (e < n && from > grid[e] + 1e-12) ++e;
            A.e_min = e;
        }
    }
    // step tables
    tab.c0.assign(n, 0.0);
    tab.c1.assign(n, 0.0);
    tab.time_true.assign(n, 0u);
    tab.disc.assign(n, 0.0);
    for (int k = 0; k < n; ++k) {
        double dt = k == 0 ? grid[0] : grid[k] - grid[k - 1];
        if (m.kind == KX_MODEL_GBM) {
            tab.c0[k] = (m.mu - 0.5 * m.sigma * m.sigma) * dt;  // simulator.rs:242
            tab.c1[k] = m.sigma * std::sqrt(dt);                 // simulator.rs:243
        } else {
            tab.c0[k] = dt;
            tab.c1[k] = std::sqrt(dt);
        }
        tab.disc[k] = std::exp(-rate * grid[k]);  // pricer.rs:353
        uint32_t bits = 0;
        for (int i = 0; i < P.n_trig; ++i)
            if (P.trig[i].cond_kind == CK_TIME && eval_time_cond(*low.time_cond[i], grid[k], low)) bits |= 1u << i;
        tab.time_true[k] = bits;
    }
    // time-only slots: first step they hold, and whether they then keep holding
    P.mono_mask = 0;
    for (int i = 0; i < P.n_trig; ++i) {
        P.first_true[i] = INT32_MAX;
        if (P.trig[i].cond_kind != CK_TIME) continue;
        int first = -1;
        bool mono = true;
        for (int k = 0; k < n; ++k) {
            const bool b = (tab.time_true[k] >> i) & 1u;
            if (b && first < 0) first = k;
            if (!b && first >= 0) mono = false;
        }
        P.first_true[i] = first < 0 ? INT32_MAX : first;
        if (mono) P.mono_mask |= 1u << i;
    }
    // next time event after step 0 for the slots armed at 0 (if none fires then)
    P.init_nte = INT32_MAX;
    const uint32_t t0 = P.root_arm & P.time_mask;
    for (int i = 0; i < P.n_trig; ++i)
        if ((t0 >> i) & 1u) P.init_nte = ((P.mono_mask >> i) & 1u) ? std::min(P.init_nte, P.first_true[i]) : 1;
}

StaticSchedule static_schedule(const KxProgram &P, const StepTables &tab) {
    StaticSchedule S;
    const int n = P.n_times;
    const int NEVER = StaticSchedule::NEVER;
    S.arm.assign(P.n_trig, NEVER);
    S.fire.assign(P.n_trig, NEVER);
    std::vector<int> parent(P.n_trig, -1);  // the when slot whose firing arms slot j
    for (int i = 0; i < P.n_trig; ++i)
        for (int j = 0; j < P.n_trig; ++j)
            if ((P.trig[i].fire_arm >> j) & 1u) parent[j] = i;
    auto first_from = [&](int i, int from) {
        for (int k = std::max(from, 0); k < n; ++k)
            if ((tab.time_true[k] >> i) & 1u) return k;
        return NEVER;
    };
    for (int i = 0; i < P.n_trig; ++i) {  // slots are numbered parents first
        const KxTrig &T = P.trig[i];
        S.arm[i] = parent[i] < 0 ? 0 : S.fire[parent[i]];
        if (T.cond_kind == CK_TIME) {
            S.fire[i] = S.arm[i] == NEVER ? NEVER : first_from(i, S.arm[i]);
        } else if (T.kind == TK_WHEN) {
            S.static_ok = false;
        }
    }
    for (int j = 0; j < P.n_leaf; ++j) {
        int acq = -1;
        for (int i = 0; i < P.n_trig; ++i)
            if (P.trig[i].kind == TK_WHEN && ((P.trig[i].leaves >> j) & 1u)) acq = i;
        const int t = acq < 0 ? 0 : S.fire[acq];
        if (t == NEVER) continue;
        bool dead = false;
        uint32_t pu = 0;
        for (int i = 0; i < P.n_trig; ++i) {
            const KxTrig &T = P.trig[i];
            if (T.kind != TK_UNTIL || !((T.leaves >> j) & 1u)) continue;
            if (T.cond_kind == CK_TIME) {
                if (S.fire[i] <= t) dead = true;  // knocked at or before the flow (pricer.rs:407-413)
            } else if (S.arm[i] != NEVER) {
                pu |= 1u << i;
            }
        }
        if (!dead) S.flows.push_back(StaticSchedule::Flow{j, t, pu});
    }
    return S;
}

}  // namespace kx
