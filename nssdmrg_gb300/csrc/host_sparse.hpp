// Host-side row-list sparse matrices, blocks and sector lists.
//
// These mirror the reference's containers: sparse_matrix / sparse_row
// (src/MATRIX/MATRIX_SPARSE.f90:28-72), sectors_list
// (src/LIST/LIST_SECTORS.f90:16-43) and block (src/BLOCKS/BLOCKS.f90:14-43).
// They hold the block-level state of a DMRG run between superblock solves;
// the superblock solve itself runs on the GPU.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <exception>
#include <map>
#include <memory>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

namespace nss {

// Host threads a parallel host loop may use, the caller's included:
// NSS_HOST_THREADS if set to a positive number (1 runs every loop on the
// calling thread), else no cap beyond each loop's own.  Read once.
inline int host_threads_cap() {
    static const int cap = [] {
        const char *e = std::getenv("NSS_HOST_THREADS");
        const int v = e ? std::atoi(e) : 0;
        return v > 0 ? v : 1 << 20;
    }();
    return cap;
}

// f0 on the calling thread and f1 on a second one (the two sides of a DMRG
// step are independent); an exception of either is rethrown after both
// have finished, f0's first.  With parallel false (work too small to pay
// for a thread, ~20 us), or when no thread can be started, both run here,
// f0 first.
template <class F0, class F1>
void run_pair(F0 &&f0, F1 &&f1, bool parallel = true) {
    std::exception_ptr e0, e1;
    std::thread th;
    if (parallel && host_threads_cap() >= 2) {
        try {
            th = std::thread([&] {
                try {
                    f1();
                } catch (...) {
                    e1 = std::current_exception();
                }
            });
        } catch (const std::system_error &) {
        }
    }
    if (!th.joinable()) {
        f0();
        f1();
        return;
    }
    try {
        f0();
    } catch (...) {
        e0 = std::current_exception();
    }
    th.join();
    if (e0) std::rethrow_exception(e0);
    if (e1) std::rethrow_exception(e1);
}

// f(i) for i in [0, n) on up to `threads` threads (the caller's among them),
// indices handed out one at a time; with parallel false, or n < 2, all run
// here in order.  If the system starts fewer threads, the ones running take
// all indices.  The first exception is rethrown after every thread ends.
template <class F>
void parallel_for(int n, F &&f, bool parallel = true, int threads = 8) {
    threads = std::min(threads, host_threads_cap());
    if (!parallel || n < 2 || threads < 2) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    const unsigned hw = std::thread::hardware_concurrency();
    const int nt = std::min(std::min(n, threads), hw > 1 ? (int)hw : 2);
    std::atomic<int> next{0};
    std::vector<std::exception_ptr> errs(nt);
    auto work = [&](int t) {
        try {
            for (int i; (i = next.fetch_add(1)) < n;) f(i);
        } catch (...) {
            errs[t] = std::current_exception();
            next.store(n);
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) {
        try {
            th.emplace_back(work, t);
        } catch (const std::system_error &) {   // no more threads: those started share the rest
            break;
        }
    }
    work(0);
    for (std::thread &x : th) x.join();
    for (const std::exception_ptr &e : errs)
        if (e) std::rethrow_exception(e);
}

// CSR matrix, 0-based.  Explicit zeros that arise from arithmetic are kept,
// as in the reference's sparse algebra.
struct Csr {
    int nrow = 0, ncol = 0;
    std::vector<int> rowptr{0};
    std::vector<int> col;
    std::vector<double> val;

    int64_t nnz() const { return (int64_t)col.size(); }
    void init(int r, int c) {
        nrow = r; ncol = c;
        rowptr.assign(r + 1, 0);
        col.clear(); val.clear();
    }
};

Csr csr_identity(int n);
Csr csr_from_dense(int nrow, int ncol, const double *a /* row-major */);
Csr csr_scale(const Csr &a, double s);
Csr csr_add(const Csr &a, const Csr &b);           // a + b
Csr csr_kron(const Csr &a, const Csr &b);           // sp_kron_matrix
// sum_t coef_t * kron(a_t, b_t) in one pass, every a_t na x na and b_t
// nb x nb: the sparse sum of the terms' Kronecker products as csr_add would
// form it (entries touched by any term are kept, also when they cancel),
// rows split over nthreads threads
struct KronTerm {
    const Csr *a, *b;
    double coef;
};
Csr csr_kron_sum(int na, int nb, const std::vector<KronTerm> &terms, int nthreads);
Csr csr_transpose(const Csr &a);                    // sp_dgr_matrix (real)
Csr csr_matmul(const Csr &a, const Csr &b);         // sp_matmul_matrix
// sp_filter_matrix_2: rows `rows`, columns `cols` (0-based state lists).
Csr csr_filter(const Csr &a, const std::vector<int> &rows, const std::vector<int> &cols);

// A QN tuple; compared with exact equality like the reference's real(8) tuples.
using Qn = std::vector<double>;

// sectors_list: QNs in first-occurrence order of the basis, ascending maps.
struct Sectors {
    std::vector<Qn> qns;
    std::vector<std::vector<int>> maps;
    std::map<Qn, int> index;
    int find(const Qn &q) const {
        auto it = index.find(q);
        return it == index.end() ? -1 : it->second;
    }
};
Sectors make_sectors(const std::vector<double> &basis, int dim, int qdim);

struct Op {
    std::string key;
    Csr m;
    std::string type;    // "bosonic" | "fermionic" | "psign"
};

struct Block {
    int length = 1;
    int dim = 1;
    int qdim = 1;
    bool fermion = false;
    std::vector<double> basis;   // dim*qdim
    std::vector<Op> ops;         // ordered as the reference's operators_list
    // rotation matrices of the renormalisations that built the block
    // (omatrices, src/BLOCKS/BLOCKS.f90:21): omats[i] belongs to length i+1,
    // omats[0] is the site's identity; shared, since the finite algorithm
    // copies blocks and never changes a stored rotation
    std::vector<std::shared_ptr<const Csr>> omats;

    Csr &op(const std::string &key);
    const Csr &op(const std::string &key) const;
    int find_op(const std::string &key) const;
    Sectors sectors() const { return make_sectors(basis, dim, qdim); }
};

}  // namespace nss
