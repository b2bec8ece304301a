// Launch-parameter table: per Chebyshev order, rows (min_points, FP32 near-field segment pairs,
// float-float segment pairs, tensor-core M2L launch form).  A plan takes the row of its order with
// the largest min_points not above its source count (make_plan); without one the defaults hold
// (2^17, 2^14, two CTAs per SM).  The rows come from the autotuner (ibim_autotune: timed matvecs
// of a prepared solve per candidate, see capi.cu), loaded from a table file (ibim_tuning_load) or
// set one by one (ibim_tuning_set).  No counterpart in the reference.
//
// The parameters change the work partition and launch shape only: the same pairs, the same MMAs,
// results equal up to the order of floating-point additions (atomic accumulation of segments).

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.cuh"

namespace ibim {

namespace {

struct Row {
    int order;
    long min_points, near, nearff;
    int form;
};

std::mutex g_mu;
std::vector<Row> g_rows;
thread_local const Tuning *g_override = nullptr;

bool valid(long near, long nearff, int form) {
    return near >= 1024 && near <= (1L << 24) && nearff >= 256 && nearff <= (1L << 22) &&
           (form == 0 || form == 2 || form == 4 || form == 6 || form == 7);
}

}  // namespace

Tuning tuning_for(int order, long npoints) {
    Tuning t;
    if (g_override) {
        t = *g_override;
    } else {
        std::lock_guard<std::mutex> lk(g_mu);
        long best = -1;
        for (const Row &r : g_rows)
            if (r.order == order && r.min_points <= npoints && r.min_points > best) {
                best = r.min_points;
                t.near_seg_pairs = r.near;
                t.nearff_seg_pairs = r.nearff;
                t.tc_form = r.form;
            }
    }
    static const int env_form = [] {
        const char *v = std::getenv("IBIM_TC_RT");
        if (!v) return -1;
        return v[0] == '4' ? 4 : v[0] == '6' ? 6 : v[0] == '7' ? 7 : v[0] == 'P' ? 0 : 2;
    }();
    if (env_form >= 0) t.tc_form = env_form;
    return t;
}

// Plans made on this thread while `t` is set use it instead of the table (the autotuner's
// candidates); nullptr restores the table.
void tuning_override(const Tuning *t) { g_override = t; }

void set_last_error(const std::string &msg);

}  // namespace ibim

using namespace ibim;

extern "C" {

int ibim_tuning_set(int order, long min_points, long near_seg_pairs, long nearff_seg_pairs, int tc_form) {
    if (order < 2 || order > 8 || min_points < 0 || !valid(near_seg_pairs, nearff_seg_pairs, tc_form)) {
        set_last_error("tuning: order in [2, 8], min_points >= 0, segment pairs in range, launch form 0, 2, 4, 6 or 7");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    for (Row &r : g_rows)
        if (r.order == order && r.min_points == min_points) {
            r = Row{order, min_points, near_seg_pairs, nearff_seg_pairs, tc_form};
            return IBIM_OK;
        }
    g_rows.push_back(Row{order, min_points, near_seg_pairs, nearff_seg_pairs, tc_form});
    return IBIM_OK;
}

int ibim_tuning_clear(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_rows.clear();
    return IBIM_OK;
}

int ibim_tuning_get(int order, long npoints, long out[3]) {
    if (!out) {
        set_last_error("tuning: null output");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    const Tuning t = tuning_for(order, npoints);
    out[0] = t.near_seg_pairs;
    out[1] = t.nearff_seg_pairs;
    out[2] = t.tc_form;
    return IBIM_OK;
}

int ibim_tuning_load(const char *path) {
    if (!path) {
        set_last_error("tuning: null path");
        return IBIM_ERR_INVALID_ARGUMENT;
    }
    std::FILE *f = std::fopen(path, "r");
    if (!f) {
        set_last_error(std::string("tuning: cannot open ") + path);
        return IBIM_ERR_IO;
    }
    std::vector<Row> rows;
    char line[512];
    int lineno = 0;
    while (std::fgets(line, sizeof line, f)) {
        ++lineno;
        const char *p = line;
        while (*p == ' ' || *p == '\t') ++p;
        if (*p == '#' || *p == '\n' || *p == '\0') continue;
        Row r{};
        if (std::sscanf(p, "%d %ld %ld %ld %d", &r.order, &r.min_points, &r.near, &r.nearff, &r.form) != 5 ||
            r.order < 2 || r.order > 8 || r.min_points < 0 || !valid(r.near, r.nearff, r.form)) {
            std::fclose(f);
            set_last_error(std::string("tuning: malformed row ") + std::to_string(lineno) + " in " + path);
            return IBIM_ERR_IO;
        }
        rows.push_back(r);
    }
    std::fclose(f);
    for (const Row &r : rows) {
        const int st = ibim_tuning_set(r.order, r.min_points, r.near, r.nearff, r.form);
        if (st != IBIM_OK) return st;
    }
    return IBIM_OK;
}

}  // extern "C"
