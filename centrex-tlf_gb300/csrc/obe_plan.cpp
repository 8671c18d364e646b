// obe_plan.cpp -- host side of prepare_lindblad_problem_py: payload validation and the
// coefficient packer that lays the expanded_sparse term list out for the GPU.
//
// Reference behaviour: rust/src/lindblad/plan.rs:1069-1308 (validation, dynamic-coefficient
// detection) and rust/src/lindblad/rhs.rs:151-384 (upper-to-packed map, term partitioning).
// The GPU layout is this project's own: terms are merged per (output, input, conjugation) into
// records whose coefficient is a *formula* (a sum of factor x coefficient products) kept in a
// per-trajectory table; records are bin-packed onto the threads of a trajectory and stored
// thread-interleaved so that each step of the gather loop is one conflict-free shared-memory
// word per thread.
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <map>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "obe_internal.h"

namespace obe {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

std::string fmt_f64(double v) {
    // Rust's Display for f64: shortest round-trip digits, positional notation.
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
    if (v == 0.0) return std::signbit(v) ? "-0" : "0";
    char buf[64];
    int prec;
    for (prec = 1; prec <= 17; ++prec) {
        std::snprintf(buf, sizeof buf, "%.*e", prec - 1, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    std::string digits;
    bool neg = false;
    const char* p = buf;
    if (*p == '-') { neg = true; ++p; }
    for (; *p && *p != 'e'; ++p)
        if (*p != '.') digits.push_back(*p);
    int exp10 = std::atoi(p + 1);
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    std::string out = neg ? "-" : "";
    int nd = static_cast<int>(digits.size());
    if (exp10 >= 0) {
        for (int i = 0; i <= exp10 || i < nd; ++i) {
            if (i == exp10 + 1) out.push_back('.');
            out.push_back(i < nd ? digits[i] : '0');
            if (i >= exp10 && i >= nd - 1) break;
        }
    } else {
        out += "0.";
        for (int i = 0; i < -exp10 - 1; ++i) out.push_back('0');
        out += digits;
    }
    return out;
}

int64_t shape_capacity(int tpt) {
    switch (tpt) {
        case 32: case 64: case 128: case 512: return static_cast<int64_t>(tpt) * 16;
        case 256: return 256 * 32;
        default: return 0;
    }
}

// Deals a plan's record lists out onto `tpt` threads of one trajectory: gather outputs (and, for
// the adjoint, input slots) longest first onto the least-loaded thread, each thread's records in
// iteration-major order (record it of thread l at it * tpt + l) ending its output with the flush
// bit; and the time-dependent formulas' products as the mixed form's product stream.
void lay_out_lanes(HostPacked& hp, int tpt) {
    const int64_t U = static_cast<int64_t>(hp.g_lane_word.size());
    auto emit = [&](const std::vector<int64_t>& ptr, const std::vector<uint32_t>& words, const std::vector<uint32_t>& lane_word,
                    std::vector<uint32_t>& recs, std::vector<uint32_t>& lane_tab, int32_t& n_iter, int32_t& n_lane) {
        std::vector<int64_t> order(U);
        std::iota(order.begin(), order.end(), 0);
        auto cost = [&](int64_t u) { return std::max<int64_t>(1, ptr[u + 1] - ptr[u]); };
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return cost(a) > cost(b); });
        std::vector<int64_t> load(tpt, 0);
        std::vector<std::vector<int64_t>> lanes(tpt);
        for (int64_t u : order) {
            const int lane = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
            lanes[lane].push_back(u);
            load[lane] += cost(u);
        }
        const int64_t iters = U > 0 ? *std::max_element(load.begin(), load.end()) : 0;
        size_t n_o = 0;
        for (auto& v : lanes) {
            std::sort(v.begin(), v.end());
            n_o = std::max(n_o, v.size());
        }
        n_iter = static_cast<int32_t>(iters);
        n_lane = static_cast<int32_t>(n_o);
        recs.assign(static_cast<size_t>(iters) * tpt, 0u);  // padding: slot 0, formula 0 (zero)
        lane_tab.assign(n_o * tpt, 0u);
        // The order of the records inside an output is free (its products are summed), so each
        // iteration picks, lane by lane, the record whose two 16-byte operands (input slot, formula
        // entry) least crowd those already chosen in the lane's quarter-warp: a 16-byte shared load
        // is served 8 lanes at a time, one wavefront per distinct address in the busiest of the 8
        // bank groups (address mod 8).  Greedy and deterministic; the iteration count does not
        // change.
        std::vector<size_t> next(tpt, 0);
        std::vector<std::vector<uint32_t>> pool(tpt);
        std::vector<uint8_t> open(tpt, 0);
        std::vector<uint32_t> seen_slot, seen_fid;
        // wavefronts of a phase after adding address a: the most distinct addresses in one bank group
        auto wavefronts = [](const std::vector<uint32_t>& seen, uint32_t a) {
            int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            bool have = false;
            for (size_t k = 0; k < seen.size(); ++k) {
                bool dup = false;
                for (size_t m = 0; m < k; ++m) dup = dup || seen[m] == seen[k];
                if (!dup) ++cnt[seen[k] & 7u];
                have = have || seen[k] == a;
            }
            if (!have) ++cnt[a & 7u];
            int mx = 0;
            for (int b = 0; b < 8; ++b) mx = cnt[b] > mx ? cnt[b] : mx;
            return mx * 16 + cnt[a & 7u];  // the phase's wavefronts, then the crowding of a's group
        };
        for (int64_t it = 0; it < iters; ++it) {
            for (int q0 = 0; q0 < tpt; q0 += 8) {
                seen_slot.clear();
                seen_fid.clear();
                for (int lane = q0; lane < q0 + 8 && lane < tpt; ++lane) {
                    uint32_t w = 0u;  // padding record: slot 0, formula 0
                    if (!open[lane] && next[lane] < lanes[lane].size()) {
                        const size_t o = next[lane]++;
                        const int64_t u = lanes[lane][o];
                        lane_tab[o * tpt + lane] = lane_word[u];
                        if (ptr[u + 1] == ptr[u]) {
                            w = kRecFlush;  // an output with no terms stays 0
                        } else {
                            pool[lane].assign(words.begin() + ptr[u], words.begin() + ptr[u + 1]);
                            open[lane] = 1;
                        }
                    }
                    if (open[lane]) {
                        auto& pl = pool[lane];
                        size_t best = 0;
                        int best_cost = 1 << 30;
                        for (size_t k = 0; k < pl.size(); ++k) {
                            const int c = wavefronts(seen_slot, pl[k] & kRecIndexMask) + wavefronts(seen_fid, pl[k] >> kRecCoefShift);
                            if (c < best_cost) { best_cost = c; best = k; }
                        }
                        w = pl[best];
                        pl.erase(pl.begin() + static_cast<std::ptrdiff_t>(best));
                        if (pl.empty()) {
                            w |= kRecFlush;
                            open[lane] = 0;
                        }
                    }
                    recs[static_cast<size_t>(it) * tpt + lane] = w;
                    seen_slot.push_back(w & kRecIndexMask);
                    seen_fid.push_back(w >> kRecCoefShift);
                }
            }
        }
    };
    emit(hp.g_ptr, hp.g_word, hp.g_lane_word, hp.rec, hp.lane_out, hp.n_iter, hp.n_out);
    emit(hp.t_ptr, hp.t_word, hp.t_lane_word, hp.trec, hp.lane_in, hp.n_titer, hp.n_tin);

    // the adjoint's parameter pass, formula-major: every formula with a product of a coefficient
    // class, followed by the records that use it (input slot, output slot, conjugate bit); the
    // formulas are dealt out longest first onto the least-loaded thread and each ends with its
    // formula entry
    {
        int64_t n = 0;
        while (n * (n + 1) / 2 < U) ++n;  // U = n (n + 1) / 2
        const int32_t F = hp.n_formula;
        std::vector<uint8_t> parametric(static_cast<size_t>(F) + 1, 0);
        for (int32_t f = 1; f <= F; ++f)
            for (int32_t q = hp.formula_ptr[f - 1]; q < hp.formula_ptr[f]; ++q)
                if (hp.prod_class[q] >= 0) parametric[f] = 1;
        std::vector<std::vector<uint32_t>> frecs(static_cast<size_t>(F) + 1);
        for (int64_t u = 0; u < U; ++u) {
            const int64_t re = static_cast<int64_t>(hp.g_lane_word[u] & 0xFFFFu);
            const uint32_t oslot = static_cast<uint32_t>(re < n ? re : n + (re - n) / 2);
            for (int64_t r = hp.g_ptr[u]; r < hp.g_ptr[u + 1]; ++r) {
                const uint32_t w = hp.g_word[r];
                const uint32_t f = w >> kRecCoefShift;
                if (f == 0 || f > static_cast<uint32_t>(F) || !parametric[f]) continue;
                uint32_t e = (w & kRecIndexMask) | (oslot << kBilOutShift);
                if (w & kRecConj) e |= kBilConj;
                frecs[f].push_back(e);
            }
        }
        std::vector<int32_t> forder;
        for (int32_t f = 1; f <= F; ++f)
            if (!frecs[f].empty()) forder.push_back(f);
        auto fcost = [&](int32_t f) {
            return static_cast<int64_t>(frecs[f].size()) + 1 + (hp.formula_ptr[f] - hp.formula_ptr[f - 1]);
        };
        std::stable_sort(forder.begin(), forder.end(), [&](int32_t a, int32_t b) { return fcost(a) > fcost(b); });
        std::vector<int64_t> bload(tpt, 0);
        std::vector<std::vector<int32_t>> lane_fs(tpt);
        for (int32_t f : forder) {
            const int lane = static_cast<int>(std::min_element(bload.begin(), bload.end()) - bload.begin());
            lane_fs[lane].push_back(f);
            bload[lane] += static_cast<int64_t>(frecs[f].size()) + 1;
        }
        const int64_t n_biter = forder.empty() ? 0 : *std::max_element(bload.begin(), bload.end());
        hp.n_biter = static_cast<int32_t>(n_biter);
        hp.bil.assign(static_cast<size_t>(n_biter) * tpt, 0u);  // padding: a record after the last formula, never closed
        for (int lane = 0; lane < tpt; ++lane) {
            int64_t it = 0;
            for (int32_t f : lane_fs[lane]) {
                for (uint32_t e : frecs[f]) hp.bil[static_cast<size_t>(it++) * tpt + lane] = e;
                hp.bil[static_cast<size_t>(it++) * tpt + lane] = kBilEnd | static_cast<uint32_t>(f);
            }
        }
    }

    // time-dependent formulas as a thread-interleaved product stream (mixed form: each thread
    // sums its formulas' products and stores the finished entries; formulas are dealt out
    // longest first onto the least-loaded thread)
    const int32_t S = hp.n_static_formula, D = hp.n_formula - hp.n_static_formula;
    auto fsize = [&](int32_t f) { return static_cast<int64_t>(hp.formula_ptr[S + f + 1] - hp.formula_ptr[S + f]); };
    std::vector<int32_t> forder(D);
    std::iota(forder.begin(), forder.end(), 0);
    std::stable_sort(forder.begin(), forder.end(), [&](int32_t a, int32_t b) { return fsize(a) > fsize(b); });
    std::vector<int64_t> fload(tpt, 0);
    std::vector<std::vector<int32_t>> lane_f(tpt);
    for (int32_t f : forder) {
        const int lane = static_cast<int>(std::min_element(fload.begin(), fload.end()) - fload.begin());
        lane_f[lane].push_back(f);
        fload[lane] += std::max<int64_t>(1, fsize(f));
    }
    const int64_t n_fiter = D > 0 ? *std::max_element(fload.begin(), fload.end()) : 0;
    hp.n_fiter = static_cast<int32_t>(n_fiter);
    hp.fstream.assign(static_cast<size_t>(n_fiter) * tpt * 4, 0u);  // padding: constant 0, no store
    for (int lane = 0; lane < tpt; ++lane) {
        int64_t it = 0;
        for (int32_t f : lane_f[lane]) {
            const uint32_t fid = static_cast<uint32_t>(1 + S + f);
            const int64_t p0 = hp.formula_ptr[S + f], len = fsize(f);
            for (int64_t q = 0; q < std::max<int64_t>(1, len); ++q) {
                uint32_t* e = &hp.fstream[(static_cast<size_t>(it) * tpt + lane) * 4];
                float fr = 0.f, fi = 0.f;
                uint32_t meta = 0u;
                if (q < len) {
                    fr = hp.prod_factor32[2 * (p0 + q)];
                    fi = hp.prod_factor32[2 * (p0 + q) + 1];
                    meta = static_cast<uint32_t>(hp.prod_class[p0 + q] + 1);
                }
                if (q + 1 >= len) meta |= kFStreamFlush | (fid << kFStreamFormulaShift);
                std::memcpy(&e[0], &fr, 4);
                std::memcpy(&e[1], &fi, 4);
                e[2] = meta;
                ++it;
            }
        }
    }
    hp.tpt = tpt;
}

int threads_per_trajectory_len(int64_t N) {
    return N <= 512 ? 32 : N <= 1024 ? 64 : N <= 2048 ? 128 : N <= 8192 ? 256 : 1024;
}

int threads_per_trajectory_for(int32_t n) {
    int64_t N = static_cast<int64_t>(n) * n;
    int t = N <= 512 ? 32 : N <= 1024 ? 64 : N <= 2048 ? 128 : N <= 8192 ? 256 : 1024;
    // OBE_TPT picks another compiled width for tuning runs, if its shape holds the state
    // (elements per trajectory: 16 per thread, 32 at 256 threads)
    if (const char* env = std::getenv("OBE_TPT")) {
        int v = std::atoi(env);
        const int64_t cap = v == 256 ? 256 * 32 : static_cast<int64_t>(v) * 16;
        if ((v == 32 || v == 64 || v == 128 || v == 256 || v == 512) && cap >= N) t = v;
    }
    return t;
}

namespace {

struct Fail {
    obe_status code;
    std::string msg;
};

[[noreturn]] void fail(obe_status code, const std::string& msg) { throw Fail{code, msg}; }

std::string strf(const char* fmt, long long a = 0, long long b = 0) {
    char buf[512];
    std::snprintf(buf, sizeof buf, fmt, a, b);
    return buf;
}

// Kind-check one expression by simulating its stack (scalar vs tuple values), the way the
// reference's compiler tracks them (ir.py:210-326), and append it to the device pool.
// Tuples may only come from tuple base slots and may only feed helpers 8, 10, 14 and 16.
DevExpr append_expr(HostPacked& hp, const obe_expr& e, int32_t n_slots, const std::vector<int32_t>& slot_is_tuple,
                    const std::vector<std::vector<double>>& tuple_grid, const std::vector<int32_t>& pchip_of_grid_slot,
                    bool allow_pchip_tables, const char* what) {
    DevExpr out{static_cast<int32_t>(hp.ins_op.size()), static_cast<int32_t>(e.n_instr)};
    std::vector<int> kinds;  // 0 scalar, 1 tuple
    std::vector<int32_t> src_slot;  // slot a stack value was loaded from (-1 otherwise)
    for (int64_t k = 0; k < e.n_instr; ++k) {
        int32_t op = e.op[k];
        int64_t idx = e.index ? e.index[k] : 0;
        int32_t argc = e.argc ? e.argc[k] : 0;
        int32_t fn = e.function ? e.function[k] : 0;
        double re = e.value ? e.value[2 * k] : 0.0, im = e.value ? e.value[2 * k + 1] : 0.0;
        int32_t dev_op = op, dev_arg = 0, dev_fn = fn;
        if (op < 1 || op > 19) fail(OBE_ERR_INVALID, strf("unknown instruction op %lld", op));
        switch (op) {
        case OP_CONST: kinds.push_back(0); src_slot.push_back(-1); break;
        case OP_SLOT:
            if (idx < 0 || idx >= n_slots)
                fail(OBE_ERR_INVALID, strf("slot index %lld out of bounds for %lld slots", idx, n_slots));
            kinds.push_back(slot_is_tuple[idx]);
            src_slot.push_back(static_cast<int32_t>(idx));
            dev_arg = static_cast<int32_t>(idx);
            break;
        case OP_TEMP: fail(OBE_ERR_UNSUPPORTED, "temporary values belong to entrywise Hamiltonian plans, which the GPU solver does not run");
        case OP_TIME: kinds.push_back(0); src_slot.push_back(-1); break;
        case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_POW:
        case OP_GT: case OP_GE: case OP_LT: case OP_LE: case OP_EQ: case OP_NE: {
            if (kinds.size() < 2) fail(OBE_ERR_INVALID, std::string("stack underflow in ") + what);
            if (kinds.back() || kinds[kinds.size() - 2])
                fail(OBE_ERR_UNSUPPORTED, std::string("elementwise tuple arithmetic is not supported by the GPU solver (") + what + ")");
            kinds.pop_back(); src_slot.pop_back();
            src_slot.back() = -1;
            break;
        }
        case OP_NEG: case OP_CONJ:
            if (kinds.empty()) fail(OBE_ERR_INVALID, std::string("stack underflow in ") + what);
            if (kinds.back()) fail(OBE_ERR_UNSUPPORTED, std::string("tuple negation/conjugation is not supported by the GPU solver (") + what + ")");
            src_slot.back() = -1;
            break;
        case OP_BUILTIN: {
            if (argc < 1 || static_cast<size_t>(argc) > kinds.size()) fail(OBE_ERR_INVALID, std::string("stack underflow in ") + what);
            if (fn < 1 || fn > 7) fail(OBE_ERR_INVALID, strf("unknown builtin function id %lld", fn));
            if (kinds[kinds.size() - argc]) fail(OBE_ERR_UNSUPPORTED, "builtin applied to a tuple");
            kinds.resize(kinds.size() - argc); src_slot.resize(src_slot.size() - argc);
            kinds.push_back(0); src_slot.push_back(-1);
            dev_arg = argc;
            break;
        }
        case OP_HELPER: {
            if (argc < 0 || static_cast<size_t>(argc) > kinds.size()) fail(OBE_ERR_INVALID, std::string("stack underflow in ") + what);
            if (argc > kMaxHelperArgs) fail(OBE_ERR_UNSUPPORTED, "helper with too many arguments");
            if (fn < 1 || fn > 16) fail(OBE_ERR_INVALID, strf("unknown helper function id %lld", fn));
            size_t base = kinds.size() - argc;
            std::vector<int> want(argc, 0);
            if (fn == 8 || fn == 10) { if (argc < 7) fail(OBE_ERR_INVALID, "multipass helper needs 7 arguments"); want[2] = want[3] = want[4] = 1; }
            if (fn == 14 || fn == 16) { if (argc < 3) fail(OBE_ERR_INVALID, "interpolation helper needs 3 arguments"); want[1] = want[2] = 1; }
            for (int32_t a = 0; a < argc; ++a)
                if (kinds[base + a] != want[a])
                    fail(OBE_ERR_UNSUPPORTED, std::string("helper argument kinds not supported by the GPU solver (") + what + ")");
            dev_arg = argc;
            if (fn == 16 && allow_pchip_tables) {
                int32_t gs = src_slot[base + 1];
                if (gs >= 0 && pchip_of_grid_slot[gs] >= 0) {
                    dev_op = OP_PCHIP_TABLE;
                    dev_fn = pchip_of_grid_slot[gs];
                }
            }
            kinds.resize(base); src_slot.resize(base);
            kinds.push_back(0); src_slot.push_back(-1);
            break;
        }
        }
        if (static_cast<int>(kinds.size()) > hp.max_stack) hp.max_stack = static_cast<int>(kinds.size());
        hp.ins_op.push_back(dev_op);
        hp.ins_arg.push_back(dev_arg);
        hp.ins_fn.push_back(dev_fn);
        hp.ins_val.push_back(re);
        hp.ins_val.push_back(im);
    }
    (void)tuple_grid;
    if (kinds.size() != 1) fail(OBE_ERR_INVALID, "expression evaluation did not end with a single stack value");
    if (kinds[0]) fail(OBE_ERR_UNSUPPORTED, std::string("tuple-valued expressions are not supported by the GPU solver (") + what + ")");
    if (hp.max_stack > kMaxStack) fail(OBE_ERR_UNSUPPORTED, "expression too deep for the GPU solver");
    return out;
}

bool uses_time(const obe_expr& e) {
    for (int64_t k = 0; k < e.n_instr; ++k)
        if (e.op[k] == OP_TIME) return true;
    return false;
}

bool uses_dynamic_slot(const obe_expr& e, const std::vector<uint8_t>& dyn_slot) {
    for (int64_t k = 0; k < e.n_instr; ++k)
        if (e.op[k] == OP_SLOT) {
            int64_t s = e.index ? e.index[k] : 0;
            if (s >= 0 && s < static_cast<int64_t>(dyn_slot.size()) && dyn_slot[s]) return true;
        }
    return false;
}

// PchipTable::from_grid_values (plan.rs:34-80)
void build_pchip(const double* grid, const double* values, int64_t n, std::vector<double>& coef) {
    if (n < 2) return;
    std::vector<double> h(n - 1), delta(n - 1), d(n);
    for (int64_t i = 0; i < n - 1; ++i) {
        h[i] = grid[i + 1] - grid[i];
        if (h[i] <= 0.0) fail(OBE_ERR_INVALID, "pchip grid must be strictly increasing");
        delta[i] = (values[i + 1] - values[i]) / h[i];
    }
    d[0] = delta[0];
    d[n - 1] = delta[n - 2];
    for (int64_t i = 1; i < n - 1; ++i) {
        bool s0 = std::signbit(delta[i - 1]), s1 = std::signbit(delta[i]);
        if (s0 != s1 || delta[i - 1] == 0.0 || delta[i] == 0.0) {
            d[i] = 0.0;
        } else {
            double w1 = 2.0 * h[i] + h[i - 1], w2 = h[i] + 2.0 * h[i - 1];
            d[i] = (w1 + w2) / (w1 / delta[i - 1] + w2 / delta[i]);
        }
    }
    for (int64_t i = 0; i < n - 1; ++i) {
        coef.push_back(values[i]);
        coef.push_back(d[i]);
        coef.push_back((3.0 * delta[i] - 2.0 * d[i] - d[i + 1]) / h[i]);
        coef.push_back((d[i] + d[i + 1] - 2.0 * delta[i]) / (h[i] * h[i]));
    }
}

int64_t upper_index(int32_t n, int32_t i, int32_t j) {
    int64_t off = 0;
    for (int32_t r = 0; r < i; ++r) off += n - r;
    return off + (j - i);
}

// ---- static-subexpression hoisting and real closure --------------------------------------
//
// The time-dependent expressions are evaluated at five stage times per step; any subtree of
// theirs that reads neither the time nor a time-dependent slot gives the same value every time.
// Such subtrees (maximal, at least two instructions, no tuples or helpers) move into new static
// compounds evaluated once per trajectory, and the expression reads them back from a new slot:
// the same operations on the same values, so results are unchanged.

struct Ins {
    int32_t op, arg, fn;
    double re, im;
};

int ins_arity(const Ins& x) {
    switch (x.op) {
    case OP_CONST: case OP_SLOT: case OP_TIME: return 0;
    case OP_NEG: case OP_CONJ: return 1;
    case OP_BUILTIN: case OP_HELPER: return x.arg;
    case OP_PCHIP_TABLE: return 3;
    default: return 2;  // arithmetic and comparisons
    }
}

std::vector<Ins> read_expr(const HostPacked& hp, const DevExpr& e) {
    std::vector<Ins> v;
    for (int32_t k = e.start; k < e.start + e.len; ++k)
        v.push_back(Ins{hp.ins_op[k], hp.ins_arg[k], hp.ins_fn[k], hp.ins_val[2 * k], hp.ins_val[2 * k + 1]});
    return v;
}

// real_ok: every instruction maps real operands to a real result in the complex VM, and the
// real-only VM reproduces that result exactly (integer powers by repeated multiplication only).
bool expr_real_closed(const std::vector<Ins>& v, const std::vector<int32_t>& slot_is_tuple) {
    for (size_t k = 0; k < v.size(); ++k) {
        const Ins& x = v[k];
        switch (x.op) {
        case OP_CONST: if (x.im != 0.0) return false; break;
        case OP_SLOT: if (x.arg < static_cast<int32_t>(slot_is_tuple.size()) && slot_is_tuple[x.arg]) return false; break;
        case OP_TIME: case OP_ADD: case OP_SUB: case OP_MUL: case OP_DIV: case OP_NEG: case OP_CONJ:
        case OP_GT: case OP_GE: case OP_LT: case OP_LE: case OP_EQ: case OP_NE: break;
        case OP_POW:
            if (k == 0 || v[k - 1].op != OP_CONST || v[k - 1].im != 0.0 || v[k - 1].re != std::rint(v[k - 1].re) ||
                std::fabs(v[k - 1].re) > 64.0)
                return false;
            break;
        case OP_BUILTIN: if (x.fn < 1 || x.fn > 7 || x.arg != 1) return false; break;
        default: return false;  // helpers, tables
        }
    }
    return true;
}

DevExpr write_expr(HostPacked& hp, const std::vector<Ins>& v, const std::vector<int32_t>& slot_is_tuple) {
    DevExpr e{static_cast<int32_t>(hp.ins_op.size()), static_cast<int32_t>(v.size()), 0, 0};
    for (const Ins& x : v) {
        hp.ins_op.push_back(x.op);
        hp.ins_arg.push_back(x.arg);
        hp.ins_fn.push_back(x.fn);
        hp.ins_val.push_back(x.re);
        hp.ins_val.push_back(x.im);
    }
    e.real_ok = expr_real_closed(v, slot_is_tuple) ? 1 : 0;
    return e;
}

// Split the hoistable subtrees out of v: returns the rewritten program and appends each
// hoisted subtree (with its new slot, numbered from next_slot) to `hoisted`.
std::vector<Ins> hoist_expr(const std::vector<Ins>& v, const std::vector<uint8_t>& dyn_slot, const std::vector<int32_t>& slot_is_tuple,
                            int32_t& next_slot, std::vector<std::pair<int32_t, std::vector<Ins>>>& hoisted) {
    const int m = static_cast<int>(v.size());
    std::vector<int> start(m), parent(m, -1);
    std::vector<uint8_t> stat(m), ok(m);
    std::vector<int> stack;
    for (int k = 0; k < m; ++k) {
        const Ins& x = v[k];
        const int a = ins_arity(x);
        bool st = x.op != OP_TIME && !(x.op == OP_SLOT && x.arg < static_cast<int32_t>(dyn_slot.size()) && dyn_slot[x.arg]);
        bool good = x.op != OP_HELPER && x.op != OP_PCHIP_TABLE &&
                    !(x.op == OP_SLOT && x.arg < static_cast<int32_t>(slot_is_tuple.size()) && slot_is_tuple[x.arg]);
        int s0 = k;
        if (a > static_cast<int>(stack.size())) return v;  // malformed: leave it alone
        for (int c = 0; c < a; ++c) {
            int ch = stack[stack.size() - a + c];
            if (c == 0) s0 = start[ch];
            st = st && stat[ch];
            good = good && ok[ch];
            parent[ch] = k;
        }
        stack.resize(stack.size() - a);
        start[k] = s0;
        stat[k] = st;
        ok[k] = good;
        stack.push_back(k);
    }
    std::vector<int> root_at(m, -1);  // subtree start -> hoisted root
    for (int k = 0; k < m; ++k) {
        const bool hoistable = stat[k] && ok[k] && k - start[k] + 1 >= 2;
        const int par = parent[k];
        if (hoistable && par >= 0 && !(stat[par] && ok[par])) root_at[start[k]] = k;
    }
    std::vector<Ins> out;
    for (int k = 0; k < m;) {
        const int r = root_at[k];
        if (r >= 0) {
            hoisted.emplace_back(next_slot, std::vector<Ins>(v.begin() + k, v.begin() + r + 1));
            out.push_back(Ins{OP_SLOT, next_slot, 0, 0.0, 0.0});
            ++next_slot;
            k = r + 1;
        } else {
            out.push_back(v[k]);
            ++k;
        }
    }
    return out;
}

}  // namespace

obe_status pack_plan(const obe_plan_desc* d, obe_plan* p) {
    try {
        if (!d) fail(OBE_ERR_INVALID, "null plan descriptor");
        if (d->n_states <= 0) fail(OBE_ERR_INVALID, "layout dimension must be positive");
        const int32_t n = d->n_states;
        p->n = n;
        p->N = static_cast<int64_t>(n) * n;
        p->U = static_cast<int64_t>(n) * (n + 1) / 2;
        p->n_slots = d->n_slots;
        p->n_base = d->n_base;
        p->n_coeff = d->n_coefficients;
        p->has_expanded = d->has_expanded;
        if (d->n_base < 0 || d->n_slots < d->n_base) fail(OBE_ERR_INVALID, "more base values than slots");
        HostPacked& hp = p->packed;

        // ---- parameter graph --------------------------------------------------------------
        std::vector<int32_t> slot_is_tuple(d->n_slots, 0);
        std::vector<std::vector<double>> tuple_grid(d->n_slots);
        hp.tuple_ptr.push_back(0);
        p->base_is_tuple.assign(d->n_base, 0);
        for (int32_t i = 0; i < d->n_base; ++i) {
            bool is_tuple = d->base_is_tuple && d->base_is_tuple[i];
            p->base_is_tuple[i] = is_tuple;
            slot_is_tuple[i] = is_tuple;
            hp.base_val.push_back(is_tuple ? 0.0 : d->base_scalar[2 * i]);
            hp.base_val.push_back(is_tuple ? 0.0 : d->base_scalar[2 * i + 1]);
            if (is_tuple) {
                hp.base_tuple.push_back(static_cast<int32_t>(hp.tuple_ptr.size()) - 1);
                for (int64_t k = d->base_tuple_ptr[i]; k < d->base_tuple_ptr[i + 1]; ++k) {
                    hp.tuple_items.push_back(d->base_tuple_items[2 * k]);
                    hp.tuple_items.push_back(d->base_tuple_items[2 * k + 1]);
                    tuple_grid[i].push_back(d->base_tuple_items[2 * k]);
                }
                hp.tuple_ptr.push_back(static_cast<int32_t>(hp.tuple_items.size() / 2));
            } else {
                hp.base_tuple.push_back(-1);
            }
        }
        // PCHIP tables and the tuple slot whose values match each table's grid exactly enough
        // for the reference's runtime match (|a - b| < 1e-15, eval.rs:590-606)
        hp.pchip_ptr.push_back(0);
        for (int32_t t = 0; t < d->n_pchip; ++t) {
            int64_t a = d->pchip_ptr[t], b = d->pchip_ptr[t + 1];
            hp.pchip_grid.insert(hp.pchip_grid.end(), d->pchip_grid + a, d->pchip_grid + b);
            hp.pchip_cptr.push_back(static_cast<int32_t>(hp.pchip_coef.size()));
            if (b - a >= 2) build_pchip(d->pchip_grid + a, d->pchip_values + a, b - a, hp.pchip_coef);
            hp.pchip_ptr.push_back(static_cast<int32_t>(hp.pchip_grid.size()));
        }
        std::vector<int32_t> pchip_of_grid_slot(d->n_slots, -1);
        for (int32_t s = 0; s < d->n_base; ++s) {
            if (!slot_is_tuple[s]) continue;
            for (int32_t t = 0; t < d->n_pchip; ++t) {
                int64_t a = d->pchip_ptr[t], b = d->pchip_ptr[t + 1];
                if (b - a != static_cast<int64_t>(tuple_grid[s].size())) continue;
                bool match = true;
                for (int64_t k = 0; k < b - a; ++k)
                    if (!(std::fabs(d->pchip_grid[a + k] - tuple_grid[s][k]) < 1e-15)) { match = false; break; }
                if (match) {
                    if (b - a < 2) break;  // a one-point table evaluates to zero; keep the direct form
                    pchip_of_grid_slot[s] = t;
                    break;
                }
            }
        }
        std::vector<uint8_t> dyn_slot(d->n_slots, 0);
        bool params_use_time = false;
        for (int32_t i = 0; i < d->n_compounds; ++i) {
            int32_t slot = d->compound_slot[i];
            if (slot < 0 || slot >= d->n_slots) fail(OBE_ERR_INVALID, strf("compound slot %lld out of bounds", slot));
            const obe_expr& e = d->compound_expr[i];
            hp.comp_slot.push_back(slot);
            hp.comp_expr.push_back(append_expr(hp, e, d->n_slots, slot_is_tuple, tuple_grid, pchip_of_grid_slot, true, "compound parameter"));
            bool dyn = uses_time(e) || uses_dynamic_slot(e, dyn_slot);
            dyn_slot[slot] = dyn;
            hp.comp_dynamic.push_back(dyn);
            params_use_time = params_use_time || uses_time(e);
        }
        if (d->n_slots > kMaxSlots) fail(OBE_ERR_UNSUPPORTED, "too many parameter slots for the GPU solver");

        // ---- decomposed coefficients (plan.rs:242-276, 1240-1291) ---------------------------
        bool ham_uses_time = false;
        for (int32_t k = 0; k < d->n_coefficients; ++k) {
            const obe_expr& e = d->coefficient_expr[k];
            hp.coeff_expr.push_back(append_expr(hp, e, d->n_slots, slot_is_tuple, tuple_grid, pchip_of_grid_slot, false, "Hamiltonian coefficient"));
            bool dyn = uses_time(e) || uses_dynamic_slot(e, dyn_slot);
            hp.coeff_dynamic.push_back(dyn);
            hp.coeff_dyn_pos.push_back(dyn ? static_cast<int32_t>(hp.dyn_ids.size()) : -1);
            if (dyn) hp.dyn_ids.push_back(k);
            ham_uses_time = ham_uses_time || uses_time(e);
        }
        p->time_dependent = params_use_time || ham_uses_time;

        // ---- hoist the static parts of the time-dependent programs -----------------------------
        {
            int32_t next_slot = d->n_slots;
            std::vector<int32_t> tuple_of(slot_is_tuple);
            std::vector<int32_t> n_comp_slot;
            std::vector<DevExpr> n_comp_expr;
            std::vector<uint8_t> n_comp_dyn;
            std::vector<std::vector<Ins>> comp_prog, coeff_prog;
            for (size_t i = 0; i < hp.comp_expr.size(); ++i) comp_prog.push_back(read_expr(hp, hp.comp_expr[i]));
            for (size_t k = 0; k < hp.coeff_expr.size(); ++k) coeff_prog.push_back(read_expr(hp, hp.coeff_expr[k]));
            hp.ins_op.clear(); hp.ins_arg.clear(); hp.ins_fn.clear(); hp.ins_val.clear();
            std::vector<std::pair<int32_t, std::vector<Ins>>> hoisted;
            for (size_t i = 0; i < comp_prog.size(); ++i) {
                std::vector<Ins> prog = comp_prog[i];
                if (hp.comp_dynamic[i]) {
                    hoisted.clear();
                    prog = hoist_expr(prog, dyn_slot, slot_is_tuple, next_slot, hoisted);
                    for (auto& hsub : hoisted) {
                        tuple_of.push_back(0);
                        n_comp_slot.push_back(hsub.first);
                        n_comp_expr.push_back(write_expr(hp, hsub.second, tuple_of));
                        n_comp_dyn.push_back(0);
                    }
                }
                n_comp_slot.push_back(hp.comp_slot[i]);
                n_comp_expr.push_back(write_expr(hp, prog, tuple_of));
                n_comp_dyn.push_back(hp.comp_dynamic[i]);
            }
            for (size_t k = 0; k < coeff_prog.size(); ++k) {
                std::vector<Ins> prog = coeff_prog[k];
                if (hp.coeff_dynamic[k]) {
                    hoisted.clear();
                    prog = hoist_expr(prog, dyn_slot, slot_is_tuple, next_slot, hoisted);
                    for (auto& hsub : hoisted) {
                        tuple_of.push_back(0);
                        n_comp_slot.push_back(hsub.first);
                        n_comp_expr.push_back(write_expr(hp, hsub.second, tuple_of));
                        n_comp_dyn.push_back(0);
                    }
                }
                coeff_prog[k] = prog;
            }
            for (size_t k = 0; k < coeff_prog.size(); ++k) hp.coeff_expr[k] = write_expr(hp, coeff_prog[k], tuple_of);
            hp.comp_slot = n_comp_slot;
            hp.comp_expr = n_comp_expr;
            hp.comp_dynamic = n_comp_dyn;
            hp.n_vm_slots = next_slot;
            hp.dyn_real_closed = 1;
            for (size_t i = 0; i < hp.comp_expr.size(); ++i)
                if (hp.comp_dynamic[i] && !hp.comp_expr[i].real_ok) hp.dyn_real_closed = 0;
            if (hp.n_vm_slots > kMaxSlots) fail(OBE_ERR_UNSUPPORTED, "too many parameter slots for the GPU solver");
        }
        if (static_cast<int>(hp.dyn_ids.size()) > kMaxDynCoeff)
            fail(OBE_ERR_UNSUPPORTED, "too many time-dependent Hamiltonian coefficients for the GPU solver");

        if (!d->has_expanded) return OBE_OK;  // solves report the missing plan

        // ---- expanded RHS validation (plan.rs:1069-1153) -----------------------------------
        const int64_t U = p->U;
        const int64_t T = d->n_terms;
        if (d->output_ptrs[0] != 0 || d->output_ptrs[U] != T)
            fail(OBE_ERR_INVALID, "expanded RHS output_ptrs must start at 0 and end at term count");
        for (int64_t u = 0; u < U; ++u)
            if (d->output_ptrs[u] > d->output_ptrs[u + 1]) fail(OBE_ERR_INVALID, "expanded RHS output_ptrs must be monotonic");
        for (int64_t t = 0; t < T; ++t) {
            if (d->input_indices[t] < 0 || d->input_indices[t] >= U)
                fail(OBE_ERR_INVALID, strf("expanded RHS input index %lld out of bounds for upper length %lld", d->input_indices[t], U));
            if (d->coeff_indices[t] >= d->n_coefficients)
                fail(OBE_ERR_INVALID, strf("expanded RHS coefficient index %lld out of bounds for %lld coefficients", d->coeff_indices[t], d->n_coefficients));
        }
        if (p->N > static_cast<int64_t>(kRecIndexMask))
            fail(OBE_ERR_UNSUPPORTED, "state too large for the GPU solver's record format (n_states <= 127)");

        // ---- upper -> packed map (rhs.rs:151-176) -------------------------------------------
        std::vector<int64_t> u_re(U), u_im(U);
        for (int32_t i = 0; i < n; ++i) { u_re[upper_index(n, i, i)] = i; u_im[upper_index(n, i, i)] = -1; }
        int64_t cursor = n;
        for (int32_t i = 0; i < n; ++i)
            for (int32_t j = i + 1; j < n; ++j) {
                int64_t u = upper_index(n, i, j);
                u_re[u] = cursor; u_im[u] = cursor + 1;
                cursor += 2;
            }

        // ---- trace preservation ------------------------------------------------------------
        // The trace is the sum of the diagonal outputs, each Re(f c^(*) v^(*)) summed over its
        // terms.  With c = a + ib (conjugated: a - ib) and v = x + iy (conjugated: x - iy), a term
        // contributes f_re a x - f_im s_c b x - f_im s_v a y - f_re s_c s_v b y (s = -1 when
        // conjugated; a static term has a = 1, b = 0).  The RHS keeps the trace for every state and
        // every coefficient value exactly when, per (input, coefficient), the four sums over the
        // diagonal outputs vanish -- up to rounding against the largest factor.
        {
            std::map<std::pair<int64_t, int64_t>, std::array<double, 4>> sums;
            double scale = 0.0;
            for (int32_t i = 0; i < n; ++i) {
                const int64_t u = upper_index(n, i, i);
                for (int64_t t = d->output_ptrs[u]; t < d->output_ptrs[u + 1]; ++t) {
                    const double fr = d->factors_re[t], fi = d->factors_im[t];
                    scale = std::max(scale, std::max(std::fabs(fr), std::fabs(fi)));
                    const double sc = d->coeff_indices[t] >= 0 && d->coeff_conj[t] ? -1.0 : 1.0;
                    const double sv = d->input_conj[t] ? -1.0 : 1.0;
                    auto& acc = sums[{d->input_indices[t], d->coeff_indices[t]}];
                    acc[0] += fr;
                    acc[1] += -fi * sc;
                    acc[2] += -fi * sv;
                    acc[3] += -fr * sc * sv;
                }
            }
            bool keeps = true;
            for (const auto& kv : sums) {
                const bool is_static = kv.first.second < 0;
                const bool diag_in = u_im[kv.first.first] < 0;
                const auto& a = kv.second;
                // a static term has no b; a diagonal input has no y
                const double resid = std::max(std::max(std::fabs(a[0]), is_static ? 0.0 : std::fabs(a[1])),
                                              std::max(diag_in ? 0.0 : std::fabs(a[2]), is_static || diag_in ? 0.0 : std::fabs(a[3])));
                if (resid > 1e-12 * scale) { keeps = false; break; }
            }
            hp.trace_preserving = keeps ? 1 : 0;
        }
        // the cost estimate's weights: per coefficient, its largest term factor
        hp.coeff_scale.assign(static_cast<size_t>(std::max<int64_t>(d->n_coefficients, 1)), 0.0);
        for (int64_t t = 0; t < T; ++t) {
            const int64_t k = d->coeff_indices[t];
            if (k >= 0)
                hp.coeff_scale[k] = std::max(hp.coeff_scale[k], std::max(std::fabs(d->factors_re[t]), std::fabs(d->factors_im[t])));
        }

        // ---- records and formulas -----------------------------------------------------------
        // A formula is the exact list of (factor, class) products of the terms merged into one
        // record; identical lists share one table entry.
        using Product = std::tuple<int32_t, double, double>;  // class, factor re, factor im
        using Formula = std::vector<Product>;
        std::map<Formula, int32_t> static_ids, dyn_ids;
        std::vector<Formula> static_list, dyn_list;
        struct Rec { int64_t in_re; bool cplx, conj; Formula f; bool dynamic; };
        std::vector<std::vector<Rec>> out_recs(U);
        for (int64_t u = 0; u < U; ++u) {
            // group the output's terms by (input, input conjugation), in input order
            std::map<std::pair<int64_t, int>, std::vector<int64_t>> groups;
            for (int64_t t = d->output_ptrs[u]; t < d->output_ptrs[u + 1]; ++t) {
                int64_t in = d->input_indices[t];
                bool diag = u_im[in] < 0;
                int conj = diag ? 0 : (d->input_conj[t] ? 1 : 0);
                groups[{u_re[in], conj}].push_back(t);
            }
            for (auto& kv : groups) {
                Rec r;
                r.in_re = kv.first.first;
                r.conj = kv.first.second != 0;
                int64_t in_upper = d->input_indices[kv.second[0]];
                r.cplx = u_im[in_upper] >= 0;
                r.dynamic = false;
                for (int64_t t : kv.second) {
                    int64_t k = d->coeff_indices[t];
                    int32_t cls = k < 0 ? -1 : static_cast<int32_t>(2 * k + (d->coeff_conj[t] ? 1 : 0));
                    r.f.emplace_back(cls, d->factors_re[t], d->factors_im[t]);
                    if (k >= 0 && hp.coeff_dynamic[k]) r.dynamic = true;
                }
                auto& ids = r.dynamic ? dyn_ids : static_ids;
                auto& lst = r.dynamic ? dyn_list : static_list;
                if (!ids.count(r.f)) { ids[r.f] = static_cast<int32_t>(lst.size()); lst.push_back(r.f); }
                out_recs[u].push_back(std::move(r));
            }
        }
        const int32_t S = static_cast<int32_t>(static_list.size());
        const int32_t D = static_cast<int32_t>(dyn_list.size());
        if (static_cast<uint32_t>(S + D) > kMaxFormulas) fail(OBE_ERR_UNSUPPORTED, "too many coefficient formulas for the GPU solver");
        hp.n_static_formula = S;
        hp.n_formula = S + D;
        hp.formula_ptr.push_back(0);
        for (int pass = 0; pass < 2; ++pass)
            for (const Formula& f : pass == 0 ? static_list : dyn_list) {
                for (const Product& pr : f) {
                    hp.prod_class.push_back(std::get<0>(pr));
                    hp.prod_factor.push_back(std::get<1>(pr));
                    hp.prod_factor.push_back(std::get<2>(pr));
                    hp.prod_factor32.push_back(static_cast<float>(std::get<1>(pr)));
                    hp.prod_factor32.push_back(static_cast<float>(std::get<2>(pr)));
                }
                hp.formula_ptr.push_back(static_cast<int32_t>(hp.prod_class.size()));
            }

        // ---- width-independent record lists ----------------------------------------------
        // gather: per output u its records (a 16-byte input slot, the formula, complex and
        // conjugate bits); the gather reads 16-byte input slots: diagonal i -> slot i, the
        // (re, im) pair at packed index r >= n -> slot n + (r - n) / 2
        auto fid_of = [&](const Rec& rc) {
            return rc.dynamic ? static_cast<uint32_t>(1 + S + dyn_ids[rc.f]) : static_cast<uint32_t>(1 + static_ids[rc.f]);
        };
        auto slot_of = [&](const Rec& rc) {
            return rc.cplx ? static_cast<uint32_t>(n + (rc.in_re - n) / 2) : static_cast<uint32_t>(rc.in_re);
        };
        hp.g_ptr.assign(U + 1, 0);
        hp.g_lane_word.assign(U, 0u);
        hp.g_word.clear();
        for (int64_t u = 0; u < U; ++u) {
            const uint32_t im = u_im[u] < 0 ? kNoImag : static_cast<uint32_t>(u_im[u]);
            hp.g_lane_word[u] = static_cast<uint32_t>(u_re[u]) | (im << 16);
            for (const Rec& rc : out_recs[u]) {
                uint32_t w = slot_of(rc) | (fid_of(rc) << kRecCoefShift);
                if (rc.cplx) w |= kRecComplex;
                if (rc.conj) w |= kRecConj;
                hp.g_word.push_back(w);
            }
            hp.g_ptr[u + 1] = static_cast<int64_t>(hp.g_word.size());
        }
        // transposed (adjoint): the same records regrouped by input slot, each reading the
        // output slot of its forward record
        {
            std::vector<std::vector<uint32_t>> in_words(U);
            hp.t_lane_word.assign(U, 0u);
            for (int64_t u = 0; u < U; ++u) {
                const uint32_t uslot = u_im[u] < 0 ? static_cast<uint32_t>(u_re[u]) : static_cast<uint32_t>(n + (u_re[u] - n) / 2);
                hp.t_lane_word[uslot] = static_cast<uint32_t>(u_re[u]) | ((u_im[u] < 0 ? kNoImag : static_cast<uint32_t>(u_im[u])) << 16);
                for (const Rec& rc : out_recs[u]) {
                    uint32_t w = uslot | (fid_of(rc) << kRecCoefShift);
                    if (rc.conj) w |= kRecConj;
                    in_words[slot_of(rc)].push_back(w);
                }
            }
            hp.t_ptr.assign(U + 1, 0);
            hp.t_word.clear();
            for (int64_t v = 0; v < U; ++v) {
                hp.t_word.insert(hp.t_word.end(), in_words[v].begin(), in_words[v].end());
                hp.t_ptr[v + 1] = static_cast<int64_t>(hp.t_word.size());
            }
        }
        if (2 * static_cast<int64_t>(p->n_coeff) + 1 > static_cast<int64_t>(kFStreamClassMask))
            fail(OBE_ERR_UNSUPPORTED, "too many Hamiltonian coefficients for the GPU solver");
        lay_out_lanes(hp, threads_per_trajectory_for(n));
        return OBE_OK;
    } catch (const Fail& f) {
        set_error(f.msg);
        return f.code;
    } catch (const std::exception& ex) {
        set_error(std::string("plan packing failed: ") + ex.what());
        return OBE_ERR_INVALID;
    }
}

}  // namespace obe

extern "C" {

const char* obe_last_error(void);

obe_status obe_plan_create(const obe_plan_desc* desc, obe_plan** out_plan) {
    if (!out_plan) {
        obe::set_error("null output pointer");
        return OBE_ERR_INVALID;
    }
    *out_plan = nullptr;
    obe_plan* p = new obe_plan();
    obe_status st = obe::pack_plan(desc, p);
    if (st != OBE_OK) {
        delete p;
        return st;
    }
    *out_plan = p;
    obe::set_error("");
    return OBE_OK;
}

int64_t obe_plan_packed_len(const obe_plan* plan) { return plan ? plan->N : 0; }
int32_t obe_plan_n_states(const obe_plan* plan) { return plan ? plan->n : 0; }

int32_t obe_plan_trace_preserving(const obe_plan* plan) { return plan ? plan->packed.trace_preserving : 0; }

int32_t obe_abi_version(void) { return OBE_ABI_VERSION; }

}  // extern "C"

namespace obe {
const char* last_error_cstr() { return g_last_error.c_str(); }
}

extern "C" const char* obe_last_error(void) { return obe::last_error_cstr(); }

// ------------------------------------------------------------------------------------------
// interpolated effective-Hamiltonian plans (rust/src/effective_lindblad/plan.rs)

namespace obe {
namespace {

using cxd = std::complex<double>;

// A parameter program evaluated on the host at t = 0 (the plan-time constant rule below): the
// scalar operations of the VM; a tuple value, a helper function or an unknown operation makes
// the program not evaluable here.
bool host_eval(const obe_expr& e, const std::vector<cxd>& slots, const std::vector<uint8_t>& is_tuple, cxd* out) {
    std::vector<cxd> st;
    for (int64_t k = 0; k < e.n_instr; ++k) {
        const int32_t op = e.op[k];
        auto pop2 = [&](cxd& l, cxd& r) {
            if (st.size() < 2) return false;
            r = st.back(); st.pop_back();
            l = st.back(); st.pop_back();
            return true;
        };
        cxd l, r;
        switch (op) {
        case 1: st.emplace_back(e.value[2 * k], e.value[2 * k + 1]); break;           // CONST
        case 2: {                                                                       // SLOT
            const int64_t s = e.index[k];
            if (s < 0 || s >= static_cast<int64_t>(slots.size()) || is_tuple[s]) return false;
            st.push_back(slots[s]);
            break;
        }
        case 4: st.emplace_back(0.0, 0.0); break;                                       // TIME
        case 5: if (!pop2(l, r)) return false; st.push_back(l + r); break;
        case 6: if (!pop2(l, r)) return false; st.push_back(l - r); break;
        case 7: if (!pop2(l, r)) return false; st.push_back(l * r); break;
        case 8: if (!pop2(l, r)) return false; st.push_back(l / r); break;
        case 9: if (!pop2(l, r)) return false; st.push_back(r == cxd(0.0, 0.0) ? cxd(1.0, 0.0) : std::exp(r * std::log(l))); break;
        case 10: if (st.empty()) return false; st.back() = -st.back(); break;           // NEG
        case 11: if (st.empty()) return false; st.back() = std::conj(st.back()); break; // CONJ
        case 12: {                                                                      // BUILTIN
            const int64_t argc = e.argc[k];
            if (argc < 1 || static_cast<int64_t>(st.size()) < argc) return false;
            const cxd v = st[st.size() - argc];
            st.resize(st.size() - argc);
            switch (e.function[k]) {
            case 1: st.push_back(std::sin(v)); break;
            case 2: st.push_back(std::cos(v)); break;
            case 3: st.push_back(std::tan(v)); break;
            case 4: st.push_back(std::exp(v)); break;
            case 5: st.emplace_back(std::abs(v), 0.0); break;
            case 6: st.emplace_back(v.real(), 0.0); break;
            case 7: st.emplace_back(v.imag(), 0.0); break;
            default: return false;
            }
            break;
        }
        case 14: case 15: case 16: case 17: case 18: case 19: {                        // comparisons
            if (!pop2(l, r)) return false;
            const double a = l.real(), b = r.real();
            const bool v = op == 14 ? a > b : op == 15 ? a >= b : op == 16 ? a < b : op == 17 ? a <= b : op == 18 ? a == b : a != b;
            st.emplace_back(v ? 1.0 : 0.0, 0.0);
            break;
        }
        default: return false;  // TEMP, HELPER, ...
        }
    }
    if (st.size() != 1) return false;
    *out = st[0];
    return true;
}

bool expr_uses_time(const obe_expr& e) {
    for (int64_t k = 0; k < e.n_instr; ++k)
        if (e.op[k] == 4) return true;
    return false;
}

// detect_constant_slot (effective_lindblad/plan.rs:205-277): a scalar base slot is its base
// value; a compound whose program reads neither the time nor a slot whose first compound reads
// the time is its value at t = 0 from the base values and the compounds before it.
bool constant_slot(const obe_plan_desc* g, int32_t slot, double* out) {
    if (slot < g->n_base && !(g->base_is_tuple && g->base_is_tuple[slot])) {
        *out = g->base_scalar[2 * slot];
        return true;
    }
    for (int32_t i = 0; i < g->n_compounds; ++i) {
        if (g->compound_slot[i] != slot) continue;
        const obe_expr& e = g->compound_expr[i];
        if (expr_uses_time(e)) return false;
        for (int64_t k = 0; k < e.n_instr; ++k) {
            if (e.op[k] != 2) continue;
            for (int32_t j = 0; j < g->n_compounds; ++j)
                if (g->compound_slot[j] == e.index[k]) {
                    if (expr_uses_time(g->compound_expr[j])) return false;
                    break;
                }
        }
        std::vector<cxd> slots(std::max(g->n_slots, 1), cxd(0.0, 0.0));
        std::vector<uint8_t> tup(slots.size(), 0);
        for (int32_t b = 0; b < g->n_base; ++b) {
            if (g->base_is_tuple && g->base_is_tuple[b]) tup[b] = 1;
            else slots[b] = cxd(g->base_scalar[2 * b], g->base_scalar[2 * b + 1]);
        }
        for (int32_t j = 0; j < g->n_compounds; ++j) {
            if (g->compound_slot[j] == slot) break;
            cxd v;
            if (host_eval(g->compound_expr[j], slots, tup, &v)) {
                slots[g->compound_slot[j]] = v;
                tup[g->compound_slot[j]] = 0;
            }
        }
        cxd v;
        if (!host_eval(e, slots, tup, &v)) return false;
        *out = v.real();
        return true;
    }
    return false;
}

}  // namespace

obe_status pack_effective(const obe_plan_desc* graph, const obe_effective_desc* eff, obe_plan* p) {
    try {
        if (!graph || !eff) fail(OBE_ERR_INVALID, "null plan descriptor");
        const int32_t n = graph->n_states;
        if (n <= 0) fail(OBE_ERR_INVALID, "layout dimension must be positive");
        if (eff->real_dim != 2 * static_cast<int64_t>(n) * n) fail(OBE_ERR_INVALID, "real_dim must be 2 n_states^2");
        if (eff->n_grid < 1 || !eff->field_grid) fail(OBE_ERR_INVALID, "field_grid length mismatch");
        for (int32_t s : {eff->field_slot, eff->rabi_slot, eff->detuning_slot})
            if (s < 0 || s >= graph->n_slots) fail(OBE_ERR_INVALID, strf("parameter slot %lld out of bounds", s));
        // the RHS reads three plan coefficients: the field slot, the Rabi rate and the detuning,
        // the latter two fixed at plan creation when the reference's constant rule applies
        double crabi = 0.0, cdet = 0.0;
        const bool rabi_const = constant_slot(graph, eff->rabi_slot, &crabi);
        const bool det_const = constant_slot(graph, eff->detuning_slot, &cdet);
        int32_t ops[3] = {2, rabi_const ? 1 : 2, det_const ? 1 : 2};
        int64_t idx[3] = {eff->field_slot, eff->rabi_slot, eff->detuning_slot};
        double vals[6] = {0.0, 0.0, crabi, 0.0, cdet, 0.0};
        int32_t zero[3] = {0, 0, 0};
        obe_expr prog[3];
        for (int k = 0; k < 3; ++k) {
            prog[k].n_instr = 1;
            prog[k].op = &ops[k];
            prog[k].index = &idx[k];
            prog[k].argc = &zero[k];
            prog[k].function = &zero[k];
            prog[k].value = &vals[2 * k];
            prog[k].scalar_only = 1;
            prog[k].output_is_tuple = 0;
        }
        obe_plan_desc d = *graph;
        d.hamiltonian_decomposed = 1;
        d.n_coefficients = 3;
        d.coefficient_expr = prog;
        d.has_expanded = 0;
        d.n_terms = 0;
        obe_status st = pack_plan(&d, p);
        if (st != OBE_OK) return st;
        HostPacked& hp = p->packed;
        const int64_t N = eff->real_dim;
        if (N > 8192) fail(OBE_ERR_UNSUPPORTED, "effective-Hamiltonian states above 8192 doubles are not supported by the GPU solver");
        p->N = N;
        p->U = N / 2;
        hp.eff = 1;
        hp.pop_stride = n + 1;
        hp.eff_grid.assign(eff->field_grid, eff->field_grid + eff->n_grid);
        for (int32_t k = 1; k < eff->n_grid; ++k)
            if (!(hp.eff_grid[k] > hp.eff_grid[k - 1])) fail(OBE_ERR_INVALID, "field_grid must be increasing");
        const obe_interp_operator* opsd[3] = {&eff->combined, &eff->optical, &eff->detuning};
        const char* names[3] = {"sparse_combined", "sparse_opt", "sparse_det"};
        hp.eff_rows.clear();
        hp.eff_cols.clear();
        hp.eff_coef.clear();
        const int64_t n_int = eff->n_grid > 1 ? eff->n_grid - 1 : 0;
        for (int k = 0; k < 3; ++k) {
            const obe_interp_operator& o = *opsd[k];
            if (!o.row_ptrs || (o.nnz > 0 && (!o.col_indices || !o.coeffs)) || o.nnz < 0 || o.nnz > (1LL << 30))
                fail(OBE_ERR_INVALID, std::string(names[k]) + ": missing or oversized arrays");
            if (o.row_ptrs[0] != 0 || o.row_ptrs[N] != o.nnz) fail(OBE_ERR_INVALID, std::string(names[k]) + ": row_ptrs must run from 0 to nnz");
            for (int64_t i = 0; i < N; ++i) {
                if (o.row_ptrs[i + 1] < o.row_ptrs[i]) fail(OBE_ERR_INVALID, std::string(names[k]) + ": row_ptrs must be monotonic");
                hp.eff_rows.push_back(static_cast<int32_t>(o.row_ptrs[i]));
            }
            hp.eff_rows.push_back(static_cast<int32_t>(o.row_ptrs[N]));
            hp.eff_nnz[k] = static_cast<int32_t>(o.nnz);
            hp.eff_col_off[k] = static_cast<int32_t>(hp.eff_cols.size());
            for (int64_t q = 0; q < o.nnz; ++q) {
                if (o.col_indices[q] < 0 || o.col_indices[q] >= N) fail(OBE_ERR_INVALID, std::string(names[k]) + ": column index out of bounds");
                hp.eff_cols.push_back(static_cast<int32_t>(o.col_indices[q]));
            }
            hp.eff_coef_off[k] = static_cast<int64_t>(hp.eff_coef.size());
            hp.eff_coef.insert(hp.eff_coef.end(), o.coeffs, o.coeffs + n_int * o.nnz * 4);
        }
        lay_out_lanes(hp, threads_per_trajectory_len(N));
        return OBE_OK;
    } catch (const Fail& f) {
        set_error(f.msg);
        return f.code;
    }
}

}  // namespace obe

extern "C" obe_status obe_effective_plan_create(const obe_plan_desc* graph, const obe_effective_desc* eff, obe_plan** out_plan) {
    if (!out_plan) {
        obe::set_error("null output pointer");
        return OBE_ERR_INVALID;
    }
    *out_plan = nullptr;
    obe_plan* p = new obe_plan();
    obe_status st = obe::pack_effective(graph, eff, p);
    if (st != OBE_OK) {
        delete p;
        return st;
    }
    *out_plan = p;
    obe::set_error("");
    return OBE_OK;
}
