// Block restart files in the reference's text format.
//
// write_block / read_block (src/BLOCKS/BLOCKS.f90:418-537): length, Dim,
// SiteType, OpName, the number of sector lists (one), the sector list
// (write_sectors_list, src/LIST/LIST_SECTORS.f90:639-669: size, qdim, then
// per sector size(qn), qn, size(map), map with 1-based states), the
// operator list (write_operators_list, src/LIST/LIST_OPERATORS.f90:602-631:
// size, then per operator key, type ("none" when empty) and the matrix) and
// the rotation-matrix list in the same layout.  A matrix is sp_write_matrix
// (src/MATRIX/MATRIX_SPARSE.f90:703-728): "Nrow Ncol", then per row its size
// followed by one "col val" record per entry, col 1-based.  All records are
// Fortran list-directed, so the reader takes whitespace-separated tokens
// (D or E exponents) and the writer prints every real with 17 significant
// digits, which a list-directed read takes back exactly.
//
// Files written by older revisions of the reference name the operators
// without the link suffix ("S_z", "S_p", "C_l1_s1", "P") and type the sign
// operator "sign"; the current code looks them up as "S_z_n", ..., "P_n"
// with type "psign" (src/DMRG_CONNECT.f90:117-146), so the reader maps
// those names.
#include "host_restart.hpp"

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <regex>
#include <sstream>
#include <stdexcept>

namespace nss {

namespace {

struct Tokens {
    std::istream &is;
    std::string next() {
        std::string t;
        if (!(is >> t)) throw std::runtime_error("read_block: unexpected end of the restart file");
        return t;
    }
    int integer() {
        const std::string t = next();
        char *end = nullptr;
        const long v = std::strtol(t.c_str(), &end, 10);
        if (end == t.c_str() || *end) throw std::runtime_error("read_block: expected an integer, got '" + t + "'");
        return (int)v;
    }
    double real() {
        std::string t = next();
        for (char &ch : t)
            if (ch == 'D' || ch == 'd') ch = 'E';
        char *end = nullptr;
        const double v = std::strtod(t.c_str(), &end);
        if (end == t.c_str() || *end) throw std::runtime_error("read_block: expected a real, got '" + t + "'");
        return v;
    }
};

std::string fmt_real(double v) {
    char buf[40];
    std::snprintf(buf, sizeof buf, "%.16E", v);   // 17 significant digits
    return buf;
}

void write_matrix(std::ostream &os, const Csr &m) {
    os << ' ' << m.nrow << ' ' << m.ncol << '\n';
    for (int i = 0; i < m.nrow; ++i) {
        os << ' ' << (m.rowptr[i + 1] - m.rowptr[i]) << '\n';
        for (int p = m.rowptr[i]; p < m.rowptr[i + 1]; ++p) os << ' ' << (m.col[p] + 1) << ' ' << fmt_real(m.val[p]) << '\n';
    }
}

Csr read_matrix(Tokens &t) {
    Csr m;
    const int nrow = t.integer(), ncol = t.integer();
    if (nrow < 0 || ncol < 0) throw std::runtime_error("read_block: negative matrix shape");
    m.init(nrow, ncol);
    for (int i = 0; i < nrow; ++i) {
        const int n = t.integer();
        if (n < 0 || n > ncol) throw std::runtime_error("read_block: bad row size");
        for (int e = 0; e < n; ++e) {
            const int c = t.integer() - 1;
            if (c < 0 || c >= ncol) throw std::runtime_error("read_block: column out of range");
            m.col.push_back(c);
            m.val.push_back(t.real());
        }
        m.rowptr[i + 1] = (int)m.col.size();
    }
    return m;
}

std::string legacy_key(const std::string &k) {
    static const std::regex legacy("^(S_z|S_p|P|C_l[0-9]+_s[0-9]+)$");
    return std::regex_match(k, legacy) ? k + "_n" : k;
}

}  // namespace

void write_block(std::ostream &os, const Block &b) {
    os << ' ' << b.length << '\n' << ' ' << b.dim << '\n';
    os << ' ' << (b.fermion ? "FERMION" : "SPIN") << '\n' << ' ' << (b.fermion ? "C" : "S") << '\n';
    os << ' ' << 1 << '\n';
    const Sectors s = b.sectors();
    os << ' ' << s.qns.size() << '\n' << ' ' << b.qdim << '\n';
    for (size_t q = 0; q < s.qns.size(); ++q) {
        os << ' ' << s.qns[q].size() << '\n';
        for (double v : s.qns[q]) os << ' ' << fmt_real(v);
        os << '\n' << ' ' << s.maps[q].size() << '\n';
        for (int st : s.maps[q]) os << ' ' << (st + 1);
        os << '\n';
    }
    os << ' ' << b.ops.size() << '\n';
    for (const Op &o : b.ops) {
        os << ' ' << o.key << '\n' << ' ' << (o.type.empty() ? "none" : o.type) << '\n';
        write_matrix(os, o.m);
    }
    os << ' ' << b.omats.size() << '\n';
    for (size_t i = 0; i < b.omats.size(); ++i) {
        os << ' ' << (i + 1) << '\n' << ' ' << "none" << '\n';
        write_matrix(os, *b.omats[i]);
    }
}

Block read_block(std::istream &is) {
    Tokens t{is};
    Block b;
    b.length = t.integer();
    b.dim = t.integer();
    std::string site = t.next();
    for (char &ch : site) ch = (char)std::toupper((unsigned char)ch);
    if (site != "SPIN" && site != "FERMION") throw std::runtime_error("read_block: unknown SiteType " + site);
    b.fermion = site == "FERMION";
    t.next();   // OpName
    if (t.integer() != 1) throw std::runtime_error("read_block: only one sector list per block is supported");
    const int nsec = t.integer();
    b.qdim = t.integer();
    if (b.dim <= 0 || b.length <= 0 || nsec <= 0 || b.qdim <= 0) throw std::runtime_error("read_block: bad header");
    b.basis.assign((size_t)b.dim * b.qdim, 0.0);
    std::vector<char> seen(b.dim, 0);
    for (int q = 0; q < nsec; ++q) {
        const int dq = t.integer();
        if (dq != b.qdim) throw std::runtime_error("read_block: QN length differs from qdim");
        std::vector<double> qn(dq);
        for (double &v : qn) v = t.real();
        const int nmap = t.integer();
        for (int e = 0; e < nmap; ++e) {
            const int st = t.integer() - 1;
            if (st < 0 || st >= b.dim || seen[st]) throw std::runtime_error("read_block: bad sector map");
            seen[st] = 1;
            for (int k = 0; k < dq; ++k) b.basis[(size_t)st * dq + k] = qn[k];
        }
    }
    for (char s : seen)
        if (!s) throw std::runtime_error("read_block: the sectors do not cover the block basis");
    const int nops = t.integer();
    for (int i = 0; i < nops; ++i) {
        Op o;
        o.key = legacy_key(t.next());
        o.type = t.next();
        if (o.type == "none") o.type.clear();
        if (o.type == "sign") o.type = "psign";
        o.m = read_matrix(t);
        if (o.m.nrow != b.dim || o.m.ncol != b.dim) throw std::runtime_error("read_block: operator " + o.key + " is not Dim x Dim");
        b.ops.push_back(std::move(o));
    }
    // the rotation list; without it (or with only "1") the block restarts a
    // run but cannot be measured, as in the reference
    std::string tok;
    if (is >> tok) {
        const int nom = std::atoi(tok.c_str());
        for (int i = 0; i < nom; ++i) {
            t.next();   // key
            t.next();   // type
            b.omats.push_back(std::make_shared<const Csr>(read_matrix(t)));
        }
    }
    return b;
}

void save_block_file(const std::string &path, const Block &b) {
    std::ofstream f(path);
    if (!f) throw std::runtime_error("save_block: cannot open " + path);
    write_block(f, b);
    if (!f) throw std::runtime_error("save_block: write failed on " + path);
}

Block load_block_file(const std::string &path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("load_block: cannot open " + path);
    return read_block(f);
}

}  // namespace nss
