// Autotuner of the mixed path's sector product.
//
// Which sectors go to the tensor-core GEMM, and with which tile width, is
// decided per shape class of superblock: N and the largest left sector
// dimension, each binned in quarter octaves.  The candidate plans are
//   0  every sector on CUDA cores (the persistent Lanczos kernel runs the
//      whole iteration in one launch),
//   1  sectors with Dl >= 32 on the tensor-core GEMM, 64-column tiles,
//   2  the same with 128-column tiles;
// candidates 1 and 2 exist only when some sector has Dl >= 32.  The first
// superblocks of a class are planned with each untried candidate in turn;
// every converged mixed solve on them records its device time per H*psi
// product, and once all are tried the class keeps the fastest.  Nothing is
// timed on the side: the measurements are the solves a run makes anyway
// (a DMRG sweep meets each class many times).  Setting NSS_TC_MIN_DL fixes
// the plan instead (tests and experiments); NSS_TC_AUTO=0 turns the tuner
// off and leaves the context's configured plan.
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <utility>

#include "device.cuh"

namespace nss {

namespace {

constexpr int NCAND = 3;

struct Entry {
    double ms_per_hv[NCAND] = {-1.0, -1.0, -1.0};
    int solves[NCAND] = {0, 0, 0};
};

std::mutex g_mu;
std::map<std::pair<int, int>, Entry> g_table;   // (device, class) -> measurements

int bin(double x) { return (int)std::floor(4.0 * std::log2(std::max(x, 1.0))); }

}  // namespace

bool tune_enabled() {
    if (std::getenv("NSS_TC_MIN_DL")) return false;
    const char *e = std::getenv("NSS_TC_AUTO");
    return !(e && std::atoi(e) == 0);
}

int tune_choose(Ctx &c, const DevSb &s, int *tc_min_dl, int *bn) {
    int maxdl = 0;
    for (int d : s.dls) maxdl = std::max(maxdl, d);
    const int cls = bin((double)s.n) * 1024 + bin((double)maxdl);
    const int ncand = maxdl >= 32 ? NCAND : 1;
    int cand = 0;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        Entry &e = g_table[{c.device, cls}];
        int untried = -1;
        for (int k = 0; k < ncand && untried < 0; ++k)
            if (e.solves[k] == 0) untried = k;
        if (untried >= 0) {
            cand = untried;
        } else {
            for (int k = 1; k < ncand; ++k)
                if (e.ms_per_hv[k] < e.ms_per_hv[cand]) cand = k;
        }
    }
    *tc_min_dl = cand == 0 ? 0 : 32;
    *bn = cand == 2 ? 128 : 64;
    c.tune_class = cls;
    c.tune_cand = cand;
    return cand;
}

void tune_record(Ctx &c, double ms, int numop) {
    if (c.tune_cand < 0 || numop <= 0 || !(ms > 0.0)) return;
    std::lock_guard<std::mutex> lk(g_mu);
    Entry &e = g_table[{c.device, c.tune_class}];
    const double x = ms / numop;
    double &m = e.ms_per_hv[c.tune_cand];
    m = (m < 0.0) ? x : std::min(m, x);
    ++e.solves[c.tune_cand];
}

int tune_lookup(int device, int cls, double *ms_per_hv, int *solves) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_table.find({device, cls});
    if (it == g_table.end()) return 0;
    for (int k = 0; k < NCAND; ++k) {
        ms_per_hv[k] = it->second.ms_per_hv[k];
        solves[k] = it->second.solves[k];
    }
    return 1;
}

void tune_reset() {
    std::lock_guard<std::mutex> lk(g_mu);
    g_table.clear();
}

}  // namespace nss
