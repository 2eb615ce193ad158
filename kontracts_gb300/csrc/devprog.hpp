// devprog.hpp — the flat program a contract is lowered to, as the kernels see it.
//
// The reference values a path by a recursive walk of the contract tree
// (cashflows, src/pricer.rs:374-418) over a materialised path. Here the tree is
// flattened once on the host into three tables that a kernel interprets while
// it steps the path forward in registers:
//
//  * triggers  — one slot per when/anytime/until node. A slot is "armed" when
//    its acquiring when-node fires (or at step 0 for top-level nodes), and from
//    then on its condition is checked every step until it is true: a when fires
//    (acquiring its sub-contract at that step: first_activation, pricer.rs:421),
//    an until knocks out (flows at or after that step are dropped,
//    pricer.rs:407-413). Pure time conditions are pre-evaluated on the grid into
//    one bit mask per step; `Spot cmp Const` is a single compare of the log-spot
//    with log(Const/s0); anything else runs a postfix expression program.
//  * flows     — one slot per one(...) leaf: its acquiring trigger, the until
//    slots above it, and the amount program (sign * product of the enclosing
//    scale observables, evaluated at the flow step as pricer.rs:391-395 does).
//  * accumulators — running max/min and window sums that Average, RunningMax
//    and RunningMin need (observable.rs:103-140), updated every step.
//
// Everything here is plain data shared by host and device code.
#pragma once
#include <stdint.h>

#define KX_MAX_TRIG 32
#define KX_MAX_LEAF 32
#define KX_MAX_ACC 8
#define KX_MAX_CODE 384
#define KX_MAX_CONST 96
#define KX_MAX_STACK 8
#define KX_MAX_AT 32

// expression opcodes (postfix, one stack of reals and booleans)
enum KxOp : uint8_t {
    OP_CONST = 0,  // push cpool[arg]
    OP_SPOT,       // push S of asset arg at the current step (arg 0 on one-asset models)
    OP_ACC,        // push value of accumulator arg
    OP_NEG,
    OP_ADD,
    OP_SUB,
    OP_MUL,
    OP_DIV,
    OP_MAX,        // f64::max / fmax: NaN-ignoring
    OP_MIN,
    OP_TRUE,
    OP_FALSE,
    OP_AT,         // push (step >= at_index[arg])
    OP_GE,
    OP_GT,
    OP_LE,
    OP_LT,
    OP_AND,        // short-circuit error semantics of `a && b` (observable.rs:164)
    OP_OR,
    OP_NOT,
};

struct KxIns {
    uint8_t op;
    uint8_t pad;
    uint16_t arg;
};

enum KxTrigKind : uint8_t { TK_WHEN = 0, TK_UNTIL = 1 };
enum KxCondKind : uint8_t { CK_TIME = 0, CK_SPOT_CMP = 1, CK_GENERAL = 2 };
enum KxCmp : uint8_t { CMP_GE = 0, CMP_GT = 1, CMP_LE = 2, CMP_LT = 3 };

struct KxTrig {
    uint8_t kind;       // KxTrigKind
    uint8_t cond_kind;  // KxCondKind
    uint8_t cmp;        // CK_SPOT_CMP: comparison of S against the constant
    uint8_t spot_slot;  // CK_SPOT_CMP: index into the bound log-threshold table
    uint16_t code_off;  // CK_GENERAL program
    uint16_t code_len;
    uint32_t fire_arm;  // TK_WHEN: trigger slots armed when this one fires
    uint32_t leaves;    // TK_WHEN: flow slots acquired when it fires;
                        // TK_UNTIL: flow slots below it (dropped from the knock on)
};

enum KxAmountKind : uint8_t { AK_CONST = 0, AK_GENERAL = 1 };

// Closed forms of the commonest AK_GENERAL amounts, evaluated inline with the
// interpreter's own operations (same result bit for bit); the result is
// negated when sign < 0.
enum KxFastAmount : uint8_t {
    FA_NONE = 0,
    FA_CALL = 1,   // max(S - K, 0)
    FA_PUT = 2,    // max(K - S, 0)
    FA_SPOT = 3,   // S
    FA_CONST = 4,  // K
};

struct KxLeaf {
    uint8_t kind;       // KxAmountKind
    uint8_t err_capable;
    uint16_t code_off;
    uint16_t code_len;
    uint8_t fast;       // KxFastAmount of an AK_GENERAL amount
    uint8_t fast_k;     // its constant K: index into cpool
    double sign;        // AK_CONST amount (+1 / -1); sign of a fast amount
};

enum KxAccKind : uint8_t { ACC_MAX = 0, ACC_MIN = 1, ACC_SUM = 2 };
enum KxInnerKind : uint8_t { IK_SPOT = 0, IK_GENERAL = 1 };

struct KxAcc {
    uint8_t kind;       // KxAccKind
    uint8_t inner;      // KxInnerKind
    uint8_t fixed;      // ACC_SUM: window end given (to_year = Some)
    uint8_t pad;        // IK_SPOT: the asset it reads (0 on one-asset models)
    uint16_t code_off;  // IK_GENERAL inner program
    uint16_t code_len;
    // bound to a grid (host fills these per launch):
    int32_t i_from;     // first step in the window
    int32_t i_to;       // last step in the window (fixed windows), else INT32_MAX
    int32_t e_min;      // earliest step it can be evaluated at without error
    int32_t static_err; // evaluating it always fails (inverted or empty fixed window)
    double inv_count;   // fixed windows: 1 / window size
};

struct KxProgram {
    int32_t n_trig, n_leaf, n_acc, n_code, n_const, n_spot_cmp, n_at;
    int32_t max_stack;
    uint32_t root_arm;     // trigger slots armed at step 0
    uint32_t root_leaves;  // flow slots acquired at step 0
    uint32_t when_mask;    // trigger slots that are when/anytime
    uint32_t until_mask;
    uint32_t time_mask;    // CK_TIME trigger slots
    uint32_t price_mask;   // CK_SPOT_CMP | CK_GENERAL trigger slots
    uint32_t all_leaves;
    uint32_t err_capable;  // some evaluation can raise MalformedContract / look-ahead
    uint32_t spot_each_step; // some accumulator or general condition reads S every step
    uint32_t simple_leaves;  // flow slots whose amount is AK_CONST or has a fast form
    KxTrig trig[KX_MAX_TRIG];
    KxLeaf leaf[KX_MAX_LEAF];
    KxAcc acc[KX_MAX_ACC];
    KxIns code[KX_MAX_CODE];
    double cpool[KX_MAX_CONST];
    // bound per launch:
    int32_t at_index[KX_MAX_AT];        // OP_AT: first step with t + 1e-12 >= date
    double spot_thr[KX_MAX_TRIG];       // CK_SPOT_CMP: log(Const / s0)
    int32_t first_true[KX_MAX_TRIG];    // CK_TIME: first step whose condition holds (INT32_MAX: never)
    uint32_t mono_mask;                 // CK_TIME slots whose condition stays true once true
    int32_t init_nte;                   // next time event after step 0 when nothing fires at t = 0
    int32_t n_times;                    // grid points (step 0 is t = 0)
};

// device-side error bits (OR-ed into one word per launch)
#define KX_ERR_MALFORMED 1u   // average window inverted or empty (observable.rs:110-130)
#define KX_ERR_LOOKAHEAD 2u   // fixed average window read before it closed
#define KX_ERR_NONFINITE 4u   // reserved
