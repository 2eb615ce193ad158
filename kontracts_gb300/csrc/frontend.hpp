// frontend.hpp — host side of the engine: serde-JSON contract parser, the
// reference's compiler (Plan + time grid), lowering to KxProgram, and binding
// of a lowered program to a grid and a model.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "../../include/kontract_gpu.h"
#include "devprog.hpp"

namespace kx {

// Thrown by host code; converted to kx_status at the C boundary. `time` and
// `step` carry the payloads of KontractError::TimeOutOfRange(f64) and
// StepOutOfRange(usize) (src/error.rs:11-15); NaN / UINT64_MAX otherwise.
struct Error {
    kx_status code;
    std::string msg;
    double time = __builtin_nan("");
    uint64_t step = UINT64_MAX;
};
[[noreturn]] void raise(kx_status code, const std::string &msg);
[[noreturn]] void raise_time_out_of_range(double t);
[[noreturn]] void raise_step_out_of_range(uint64_t step);

// ---- AST (src/ast.rs:34-206) ------------------------------------------------
enum class NK {
    // contracts
    Zero, One, Give, CAnd, COr, Scale, When, Anytime, Until,
    // conditions
    Bool, At, Ge, Gt, Le, Lt, And, Or, Not,
    // observables
    Const, Spot, Neg, Add, Sub, Mul, Div, Max, Min, Average, RunningMax, RunningMin,
};

struct Node {
    NK k;
    double num = 0.0;        // Const value, At date
    bool flag = false;       // Bool value
    std::string text;        // One currency, Spot asset
    bool has_from = false, has_to = false;
    double from = 0.0, to = 0.0;  // Average window
    std::vector<std::unique_ptr<Node>> kid;
};
using NodeP = std::unique_ptr<Node>;

NodeP parse_contract_json(const char *json);

// ---- compiler (src/compiler.rs) ---------------------------------------------
struct Plan {
    std::vector<std::string> assets;  // sorted, unique
    std::vector<double> fixed_dates;  // sorted, deduplicated within 1e-12
    double horizon = 0.0;
    bool needs_fine_grid = false;
};
Plan compile_plan(const Node &contract);
std::vector<double> sort_dedup(std::vector<double> v);
std::vector<double> time_grid_forced(const Plan &p, uint32_t steps_per_year, bool force_fine);

// ---- lowering ---------------------------------------------------------------
struct SpotCmp {
    double c;  // the constant S is compared with
};
struct AccWindow {
    bool has_from = false, has_to = false;
    double from = 0.0, to = 0.0;
};

struct Lowered {
    KxProgram prog;                      // model/grid independent part filled
    std::vector<double> at_dates;        // OP_AT slot -> date
    std::vector<SpotCmp> spot_cmp;       // CK_SPOT_CMP slot -> constant
    std::vector<const Node *> time_cond; // trigger slot -> condition (CK_TIME only)
    std::vector<AccWindow> acc_window;   // accumulator slot -> window
    std::vector<std::string> spot_assets;// assets named by Spot(...) in the program
    bool has_running_average = false;
};

struct Program {  // what kx_program points at
    NodeP ast;
    Plan plan;
    Lowered low;
    std::string json;
    // The reference parses in Contract::from_json but only compiles inside
    // price_gbm (pricer.rs:102), so compile/lowering errors are kept here and
    // raised by the calls that need the plan or the lowered table.
    kx_status plan_status = KX_OK, low_status = KX_OK;
    std::string plan_msg, low_msg;
    void check(bool need_lowered) const {
        if (plan_status != KX_OK) raise(plan_status, plan_msg);
        if (need_lowered && low_status != KX_OK) raise(low_status, low_msg);
    }
};

void lower(Program &p);

// ---- binding to a grid and a model -----------------------------------------
struct Model {
    int kind = KX_MODEL_GBM;
    int scheme = KX_HESTON_REFERENCE_FLOOR;
    double s0 = 100, mu = 0, sigma = 0.2;
    double v0 = 0.04, kappa = 1, theta = 0.04, sigma_v = 0, rho = 0, r = 0;
    std::string asset = "ASSET";
    // KX_MODEL_MULTI_GBM (CorrelatedGbmN, multi_asset.rs:49-105): the factors'
    // names, spots, drifts and volatilities, and the packed lower Cholesky
    // factor of their correlation (row i: chol[i (i + 1) / 2 + j], j <= i)
    std::vector<std::string> assets;
    std::vector<double> a_s0, a_mu, a_sigma, chol;
    bool requires_fine_grid() const { return kind == KX_MODEL_HESTON; }
    int draws_per_step() const {
        return kind == KX_MODEL_HESTON ? 2 : kind == KX_MODEL_MULTI_GBM ? (int)assets.size() : 1;
    }
};
Model model_from_c(const kx_model *m);
void validate_model(const Model &m);
void validate_grid(const std::vector<double> &g);

// Per-step record the kernels load every step (grid step k >= 1).
// GBM:    c0 = (mu - sigma^2/2) dt, c1 = sigma sqrt(dt)
// Heston: c0 = dt,                  c1 = sqrt(dt)
struct StepTables {
    std::vector<double> c0, c1;
    std::vector<uint32_t> time_true;  // CK_TIME trigger bits true at step k
    std::vector<double> disc;         // exp(-rate * t_k)
};

// Fill the grid-dependent fields of `out` (a copy of low.prog) and the step
// tables for `grid`, model `m` and discount `rate`.
void bind(const Lowered &low, const std::vector<double> &grid, const Model &m, double rate,
          KxProgram &out, StepTables &tab);

// Static schedule of a bound program whose when/anytime conditions depend on
// time only: every slot's arming and firing step is then path-independent.
// until slots with price conditions are listed in `price_untils` (their
// arming step is static too); time-only untils knock at a static step.
struct StaticSchedule {
    static constexpr int NEVER = 0x7fffffff;
    std::vector<int> arm, fire;        // per trigger slot (fire = knock step for untils)
    struct Flow {
        int leaf;
        int step;                      // the flow date (grid index)
        uint32_t price_untils;         // price-condition until slots above the flow
    };
    std::vector<Flow> flows;           // flows that are paid (not knocked by a time-only until)
    bool static_ok = true;             // false if some when/anytime condition reads prices
};
StaticSchedule static_schedule(const KxProgram &P, const StepTables &tab);

}  // namespace kx
