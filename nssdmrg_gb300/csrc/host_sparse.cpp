// Host CSR algebra, sector lists and blocks (see host_sparse.hpp).
#include "host_sparse.hpp"

#include <algorithm>
#include <stdexcept>

namespace nss {

Csr csr_identity(int n) {
    Csr a;
    a.init(n, n);
    a.col.resize(n);
    a.val.assign(n, 1.0);
    for (int i = 0; i < n; ++i) {
        a.rowptr[i + 1] = i + 1;
        a.col[i] = i;
    }
    return a;
}

Csr csr_from_dense(int nrow, int ncol, const double *d) {
    Csr a;
    a.init(nrow, ncol);
    for (int i = 0; i < nrow; ++i) {
        for (int j = 0; j < ncol; ++j) {
            double v = d[(size_t)i * ncol + j];
            if (v != 0.0) {
                a.col.push_back(j);
                a.val.push_back(v);
            }
        }
        a.rowptr[i + 1] = (int)a.col.size();
    }
    return a;
}

Csr csr_scale(const Csr &a, double s) {
    Csr c = a;
    for (double &v : c.val) v *= s;
    return c;
}

// Row-wise merge with a dense scatter accumulator; entries present in either
// operand are kept (also when they cancel), like sp_sum in the reference.
Csr csr_add(const Csr &a, const Csr &b) {
    if (a.nrow != b.nrow || a.ncol != b.ncol) throw std::runtime_error("csr_add: shape mismatch");
    Csr c;
    c.init(a.nrow, a.ncol);
    std::vector<int> pos(a.ncol, -1);
    c.col.reserve(a.col.size() + b.col.size());
    c.val.reserve(a.col.size() + b.col.size());
    for (int i = 0; i < a.nrow; ++i) {
        int start = (int)c.col.size();
        for (const Csr *m : {&a, &b}) {
            for (int jj = m->rowptr[i]; jj < m->rowptr[i + 1]; ++jj) {
                int j = m->col[jj];
                if (pos[j] < 0) {
                    pos[j] = (int)c.col.size();
                    c.col.push_back(j);
                    c.val.push_back(m->val[jj]);
                } else {
                    c.val[pos[j]] += m->val[jj];
                }
            }
        }
        for (int jj = start; jj < (int)c.col.size(); ++jj) pos[c.col[jj]] = -1;
        c.rowptr[i + 1] = (int)c.col.size();
    }
    return c;
}

// sp_kron_matrix (src/MATRIX/MATRIX_SPARSE.f90:832-876): row i*B.nrow+k,
// column j*B.ncol+l.
Csr csr_kron(const Csr &a, const Csr &b) {
    Csr c;
    c.init(a.nrow * b.nrow, a.ncol * b.ncol);
    c.col.reserve((size_t)a.nnz() * b.nnz());
    c.val.reserve((size_t)a.nnz() * b.nnz());
    for (int i = 0; i < a.nrow; ++i)
        for (int k = 0; k < b.nrow; ++k) {
            for (int ia = a.rowptr[i]; ia < a.rowptr[i + 1]; ++ia)
                for (int kb = b.rowptr[k]; kb < b.rowptr[k + 1]; ++kb) {
                    c.col.push_back(b.col[kb] + a.col[ia] * b.ncol);
                    c.val.push_back(a.val[ia] * b.val[kb]);
                }
            c.rowptr[i * b.nrow + k + 1] = (int)c.col.size();
        }
    return c;
}

Csr csr_kron_sum(int na, int nb, const std::vector<KronTerm> &terms, int nthreads) {
    for (const KronTerm &t : terms)
        if (t.a->nrow != na || t.a->ncol != na || t.b->nrow != nb || t.b->ncol != nb)
            throw std::runtime_error("csr_kron_sum: term shape mismatch");
    const int n = na * nb;
    nthreads = std::max(1, std::min(nthreads, na));
    struct Part {
        std::vector<int> rowlen, col;
        std::vector<double> val;
    };
    std::vector<Part> parts(nthreads);
    auto work = [&](int ti) {
        Part &P = parts[ti];
        const int i0 = (int)((int64_t)na * ti / nthreads), i1 = (int)((int64_t)na * (ti + 1) / nthreads);
        std::vector<int> pos(n, -1);
        P.rowlen.reserve((size_t)(i1 - i0) * nb);
        for (int i = i0; i < i1; ++i)
            for (int k = 0; k < nb; ++k) {
                const int start = (int)P.col.size();
                for (const KronTerm &t : terms) {
                    const Csr &a = *t.a, &b = *t.b;
                    for (int ia = a.rowptr[i]; ia < a.rowptr[i + 1]; ++ia) {
                        const int cbase = a.col[ia] * nb;
                        const double av = a.val[ia];
                        for (int kb = b.rowptr[k]; kb < b.rowptr[k + 1]; ++kb) {
                            const int j = cbase + b.col[kb];
                            const double v = (av * b.val[kb]) * t.coef;
                            if (pos[j] < 0) {
                                pos[j] = (int)P.col.size();
                                P.col.push_back(j);
                                P.val.push_back(v);
                            } else {
                                P.val[pos[j]] += v;
                            }
                        }
                    }
                }
                for (int jj = start; jj < (int)P.col.size(); ++jj) pos[P.col[jj]] = -1;
                P.rowlen.push_back((int)P.col.size() - start);
            }
    };
    // the row ranges on threads (parallel_for: exceptions reach the caller,
    // parts no thread takes run here); assembled below in row order
    parallel_for(nthreads, work, nthreads > 1, nthreads);
    Csr c;
    c.init(n, n);
    size_t nnz = 0;
    for (const Part &P : parts) nnz += P.col.size();
    c.col.reserve(nnz);
    c.val.reserve(nnz);
    int r = 0;
    for (const Part &P : parts) {
        for (int len : P.rowlen) {
            c.rowptr[r + 1] = c.rowptr[r] + len;
            ++r;
        }
        c.col.insert(c.col.end(), P.col.begin(), P.col.end());
        c.val.insert(c.val.end(), P.val.begin(), P.val.end());
    }
    return c;
}

// sp_dgr_matrix (src/MATRIX/MATRIX_SPARSE.f90:1063-1113), real case.
Csr csr_transpose(const Csr &a) {
    Csr c;
    c.init(a.ncol, a.nrow);
    std::vector<int> cnt(a.ncol + 1, 0);
    for (int j : a.col) cnt[j + 1]++;
    for (int j = 0; j < a.ncol; ++j) cnt[j + 1] += cnt[j];
    c.rowptr = cnt;
    c.col.resize(a.col.size());
    c.val.resize(a.col.size());
    std::vector<int> next(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < a.nrow; ++i)
        for (int jj = a.rowptr[i]; jj < a.rowptr[i + 1]; ++jj) {
            int p = next[a.col[jj]]++;
            c.col[p] = i;
            c.val[p] = a.val[jj];
        }
    return c;
}

// sp_matmul_matrix (src/MATRIX/MATRIX_SPARSE.f90:931-1024): row-by-row
// Gustavson product with a dense accumulator.
Csr csr_matmul(const Csr &a, const Csr &b) {
    if (a.ncol != b.nrow) throw std::runtime_error("csr_matmul: shape mismatch");
    Csr c;
    c.init(a.nrow, b.ncol);
    std::vector<int> pos(b.ncol, -1);
    for (int i = 0; i < a.nrow; ++i) {
        int start = (int)c.col.size();
        for (int ia = a.rowptr[i]; ia < a.rowptr[i + 1]; ++ia) {
            int k = a.col[ia];
            double av = a.val[ia];
            for (int kb = b.rowptr[k]; kb < b.rowptr[k + 1]; ++kb) {
                int j = b.col[kb];
                if (pos[j] < 0) {
                    pos[j] = (int)c.col.size();
                    c.col.push_back(j);
                    c.val.push_back(av * b.val[kb]);
                } else {
                    c.val[pos[j]] += av * b.val[kb];
                }
            }
        }
        for (int jj = start; jj < (int)c.col.size(); ++jj) pos[c.col[jj]] = -1;
        c.rowptr[i + 1] = (int)c.col.size();
    }
    return c;
}

// sp_filter_matrix_2 (src/MATRIX/MATRIX_SPARSE.f90:560-628): keep rows
// `rows` and columns in `cols`, renumbered by their position in `cols`.
Csr csr_filter(const Csr &a, const std::vector<int> &rows, const std::vector<int> &cols) {
    Csr c;
    c.init((int)rows.size(), (int)cols.size());
    std::vector<int> local(a.ncol, -1);
    for (int j = 0; j < (int)cols.size(); ++j) local[cols[j]] = j;
    for (int r = 0; r < (int)rows.size(); ++r) {
        int i = rows[r];
        for (int jj = a.rowptr[i]; jj < a.rowptr[i + 1]; ++jj) {
            int js = local[a.col[jj]];
            if (js < 0) continue;
            c.col.push_back(js);
            c.val.push_back(a.val[jj]);
        }
        c.rowptr[r + 1] = (int)c.col.size();
    }
    return c;
}

// construct_sectors_tbasis / put_sectors_list (src/LIST/LIST_SECTORS.f90:
// 128-217): QNs in first-occurrence order; maps are ascending.
Sectors make_sectors(const std::vector<double> &basis, int dim, int qdim) {
    Sectors s;
    for (int i = 0; i < dim; ++i) {
        Qn q(basis.begin() + (size_t)i * qdim, basis.begin() + (size_t)(i + 1) * qdim);
        auto it = s.index.find(q);
        if (it == s.index.end()) {
            s.index.emplace(q, (int)s.qns.size());
            s.qns.push_back(q);
            s.maps.push_back({i});
        } else {
            s.maps[it->second].push_back(i);
        }
    }
    return s;
}

int Block::find_op(const std::string &key) const {
    for (size_t i = 0; i < ops.size(); ++i)
        if (ops[i].key == key) return (int)i;
    return -1;
}

Csr &Block::op(const std::string &key) {
    int i = find_op(key);
    if (i < 0) throw std::runtime_error("block operator not found: " + key);
    return ops[i].m;
}

const Csr &Block::op(const std::string &key) const {
    int i = find_op(key);
    if (i < 0) throw std::runtime_error("block operator not found: " + key);
    return ops[i].m;
}

}  // namespace nss
