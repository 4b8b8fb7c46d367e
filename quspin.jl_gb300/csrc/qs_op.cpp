// qs_op.cpp -- QuantumLinearOperator construction (host side).
//
// Restates the host logic of QuantumLinearOperator(basis, static_list; ...)
// (src/operators.jl:2492-2552): term consolidation (_consolidate_terms,
// 214-263), the structural Hermitian test (_structured_is_hermitian,
// 2979-3007), check_pcon (src/discrete_basis.jl:2333-2339), dtype promotion
// (_coefficient_type, 329-341) and the diagonal extraction of structurally
// diagonal terms (2348-2429).  The reference's check_symm builds dense parent
// matrices; here it is the structural equivalent: every generator of the
// symmetry group, acting on sites (and flipping +/- and the sign of z/y on
// flipped sites), must map the consolidated term set onto itself.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "qs_internal.h"

namespace qs {

namespace {

using cd = std::complex<double>;

struct Coupling {
    cd coef;
    std::vector<int> sites;  // one-based
};
struct Term {
    std::string op;
    std::vector<Coupling> couplings;
};

bool is_diag_op(const std::string& op) {
    for (char c : op)
        if (c != 'I' && c != 'z' && c != 'n' && c != '|') return false;
    return true;
}

// _consolidate_terms: sum duplicate (op, sites) in first-seen order, drop zeros.
std::vector<Term> consolidate(const std::vector<Term>& terms) {
    std::map<std::pair<std::string, std::vector<int>>, cd> coeffs;
    std::vector<std::pair<std::string, std::vector<int>>> order;
    for (const Term& t : terms)
        for (const Coupling& c : t.couplings) {
            auto key = std::make_pair(t.op, c.sites);
            auto it = coeffs.find(key);
            if (it == coeffs.end()) {
                order.push_back(key);
                coeffs[key] = c.coef;
            } else {
                it->second += c.coef;
            }
        }
    std::vector<Term> out;
    std::map<std::string, size_t> where;
    for (const auto& key : order) {
        cd c = coeffs[key];
        if (c == cd(0, 0)) continue;
        auto it = where.find(key.first);
        if (it == where.end()) {
            where[key.first] = out.size();
            out.push_back(Term{key.first, {}});
            it = where.find(key.first);
        }
        out[it->second].couplings.push_back(Coupling{c, key.second});
    }
    return out;
}

bool structured_hermitian(const std::vector<Term>& terms) {
    std::map<std::pair<std::string, std::vector<int>>, cd> coeffs;
    for (const Term& t : terms)
        for (const Coupling& c : t.couplings) coeffs[std::make_pair(t.op, c.sites)] += c.coef;
    for (const auto& kv : coeffs) {
        std::string adj = kv.first.first;
        for (char& ch : adj) {
            if (ch == '+') ch = '-';
            else if (ch == '-') ch = '+';
        }
        auto it = coeffs.find(std::make_pair(adj, kv.first.second));
        if (it == coeffs.end()) return false;
        cd a = it->second, b = std::conj(kv.second);
        double tol = std::max(3e-12, 3e-12 * std::max(std::abs(a), std::abs(b)));
        if (std::abs(a - b) > tol) return false;
    }
    return true;
}

// Canonical key of one coupling after a group element acts on it: (site, op)
// pairs stably sorted by site (operators on different sites commute; the
// order on a repeated site is kept), plus the coefficient sign picked up by
// flipped z / y operators.
struct Canon {
    std::vector<std::pair<int, char>> ops;
    bool operator<(const Canon& o) const { return ops < o.ops; }
};

std::map<Canon, cd> canonical_set(const std::vector<Term>& terms, int L, int refl, int shift, uint64_t mask,
                                  const std::vector<int>* perm = nullptr) {
    std::map<Canon, cd> out;
    for (const Term& t : terms)
        for (const Coupling& c : t.couplings) {
            Canon k;
            cd coef = c.coef;
            for (size_t i = 0; i < t.op.size(); ++i) {
                int b = c.sites[i] - 1;
                int nb = refl ? (L - 1 - b) : b;
                nb = ((nb + shift) % L + L) % L;
                if (perm) nb = (*perm)[b];   // a general site map
                char ch = t.op[i];
                if ((mask >> nb) & 1ull) {
                    if (ch == '+') ch = '-';
                    else if (ch == '-') ch = '+';
                    else if (ch == 'z' || ch == 'y') coef = -coef;
                }
                k.ops.push_back(std::make_pair(nb, ch));
            }
            std::stable_sort(k.ops.begin(), k.ops.end(),
                             [](const std::pair<int, char>& a, const std::pair<int, char>& b) { return a.first < b.first; });
            out[k] += coef;
        }
    return out;
}

bool same_sets(const std::map<Canon, cd>& a, const std::map<Canon, cd>& b) {
    auto close = [](cd x, cd y) { return std::abs(x - y) <= 1e-10 * std::max(1.0, std::max(std::abs(x), std::abs(y))); };
    for (const auto& kv : a) {
        auto it = b.find(kv.first);
        cd other = it == b.end() ? cd(0, 0) : it->second;
        if (!close(kv.second, other)) return false;
    }
    for (const auto& kv : b) {
        auto it = a.find(kv.first);
        cd other = it == a.end() ? cd(0, 0) : it->second;
        if (!close(kv.second, other)) return false;
    }
    return true;
}

bool commutes_with_group(const Basis& b, const std::vector<Term>& terms) {
    if (!b.symmetric) return true;
    auto base = canonical_set(terms, b.L, 0, 0, 0);
    for (const Generator& g : b.gens) {
        auto img = canonical_set(terms, b.L, g.refl, g.shift, g.mask, g.kind == GEN_GENERAL ? &g.perm : nullptr);
        if (!same_sets(base, img)) return false;
    }
    return true;
}

// Transition program of one coupling.  `transposed_chain`: the chain of A^T
// (characters in string order, + <-> -, y -> -y); otherwise A's own chain
// (characters right to left, src/operators.jl:2571-2577).
TermProg make_prog(const std::string& op, const Coupling& c, bool transposed_chain, int pauli) {
    TermProg p;
    std::memset(&p, 0, sizeof(p));
    int n = (int)op.size();
    p.nops = n;
    cd coef = c.coef;
    for (int i = 0; i < n; ++i) {
        int src = transposed_chain ? i : (n - 1 - i);
        char ch = op[src];
        if (transposed_chain) {
            if (ch == '+') ch = '-';
            else if (ch == '-') ch = '+';
            else if (ch == 'y') coef = -coef;
        }
        p.ops[i] = ch;
        p.sites[i] = (int8_t)(c.sites[src] - 1);
    }
    p.coef_re = coef.real();
    p.coef_im = coef.imag();
    // compiled form for distinct sites
    uint64_t seen = 0;
    bool distinct = true;
    for (int i = 0; i < n; ++i) {
        uint64_t bit = 1ull << p.sites[i];
        if (seen & bit) distinct = false;
        seen |= bit;
    }
    p.distinct = distinct ? 1 : 0;
    if (distinct) {
        const double zs = pauli ? 1.0 : 0.5, pm = pauli ? 2.0 : 1.0;
        cd amp = coef;
        for (int i = 0; i < n; ++i) {
            uint64_t bit = 1ull << p.sites[i];
            switch (p.ops[i]) {
                case 'I': break;
                case 'z': p.zmask |= bit; amp *= zs; break;
                case '+': p.need0 |= bit; p.flip |= bit; amp *= pm; break;
                case '-': p.need1 |= bit; p.flip |= bit; amp *= pm; break;
                case 'x': p.flip |= bit; amp *= zs; break;
                case 'y': p.flip |= bit; p.ymask |= bit; amp *= cd(0, zs); break;
                default: break;
            }
        }
        p.amp0_re = amp.real();
        p.amp0_im = amp.imag();
    }
    return p;
}

}  // namespace

Op* op_create(Basis* basis, const qs_term* terms, int nterms, const double* diagonal, int checks) {
    const Basis& b = *basis;
    if (nterms < 0) throw Error(QS_ERR_ARGUMENT, "nterms must be nonnegative");
    std::vector<Term> pub;
    bool complex_coef = false;
    for (int t = 0; t < nterms; ++t) {
        const qs_term& q = terms[t];
        if (!q.op || !q.op[0]) throw Error(QS_ERR_ARGUMENT, "operator string cannot be empty");
        std::string op(q.op);
        int arity = 0;
        for (char ch : op) {
            if (ch == '|') continue;
            ++arity;
            if (ch != 'I' && ch != 'z' && ch != '+' && ch != '-' && ch != 'x' && ch != 'y')
                throw Error(QS_ERR_ARGUMENT, std::string("unsupported spin operator '") + ch + "'");
        }
        if ((int)op.size() != arity) throw Error(QS_ERR_ARGUMENT, "unsupported spin operator '|'");
        if (arity > kMaxOps) throw Error(QS_ERR_UNSUPPORTED, "operator strings longer than 8 characters");
        if (q.complex_coeffs) complex_coef = true;
        Term T{op, {}};
        for (int c = 0; c < q.n_couplings; ++c) {
            Coupling cp;
            cp.coef = cd(q.coeffs[2 * c], q.coeffs[2 * c + 1]);
            for (int i = 0; i < arity; ++i) {
                int site = q.sites[c * arity + i];
                if (site < 1 || site > b.L)
                    throw Error(QS_ERR_ARGUMENT, "site " + std::to_string(site) + " lies outside 1:" + std::to_string(b.L));
                cp.sites.push_back(site);
            }
            T.couplings.push_back(cp);
        }
        pub.push_back(T);
    }
    std::vector<Term> checked = consolidate(pub);
    bool herm = structured_hermitian(checked);
    if ((checks & QS_CHECK_HERM) && !herm) throw Error(QS_ERR_ARGUMENT, "operator list is not Hermitian");
    if ((checks & QS_CHECK_PCON) && b.nup >= 0) {
        for (const Term& t : checked) {
            int change = 0;
            for (char ch : t.op) {
                if (ch == 'x' || ch == 'y') change = 1 << 20;
                if (ch == '+') ++change;
                if (ch == '-') --change;
            }
            if (change != 0) throw Error(QS_ERR_ARGUMENT, "operator list violates the selected particle sector");
        }
    }
    bool commuting = commutes_with_group(b, checked);
    if ((checks & QS_CHECK_SYMM) && !commuting)
        throw Error(QS_ERR_ARGUMENT, "operator list violates the selected symmetry sector");

    Op* op = new Op();
    op->basis = basis;
    if (cudaGetDevice(&op->device) != cudaSuccess) {
        cudaGetLastError();
        delete op;
        throw Error(QS_ERR_CUDA, "no current CUDA device");
    }
    bool has_y = false;
    for (const Term& t : checked)
        if (t.op.find('y') != std::string::npos) has_y = true;
    op->complex_mat = complex_coef || has_y || b.complex_chars || (diagonal && (checks & QS_DIAG_COMPLEX));
    op->commuting = commuting;
    op->extracted = commuting;
    if (diagonal) {
        op->user_diag.resize(b.n);
        for (int64_t i = 0; i < b.n; ++i) op->user_diag[i] = cd(diagonal[2 * i], diagonal[2 * i + 1]);
        if (checks & QS_CHECK_HERM)
            for (int64_t i = 0; i < b.n; ++i)
                if (diagonal[2 * i + 1] != 0.0) {
                    delete op;
                    throw Error(QS_ERR_ARGUMENT, "a Hermitian operator requires a real diagonal");
                }
    }
    bool diag_real = true;
    for (int64_t i = 0; i < (int64_t)op->user_diag.size(); ++i)
        if (op->user_diag[i].imag() != 0.0) diag_real = false;
    op->hermitian = (checks & QS_CHECK_HERM) ? true : (herm && diag_real);
    if (b.dense_proj) {
        // P^H A P from the operator on the parent sector (qs_projector.cu)
        try {
            QS_CUDA(cudaStreamCreateWithFlags(&op->own_stream, cudaStreamNonBlocking));
            op->stream = op->own_stream;
            op->commuting = false;
            op->extracted = false;
            op_build_dense(*op, terms, nterms, checks);
        } catch (...) {
            delete op;
            throw;
        }
        return op;
    }
    std::vector<TermProg> fwd, bwd;
    for (const Term& t : checked) {
        bool diag = is_diag_op(t.op);
        for (const Coupling& c : t.couplings) {
            if (diag && op->extracted) {
                op->diag_progs.push_back(make_prog(t.op, c, false, b.spec.pauli));
            } else {
                fwd.push_back(make_prog(t.op, c, true, b.spec.pauli));
                bwd.push_back(make_prog(t.op, c, false, b.spec.pauli));
            }
        }
    }
    op->progs = fwd;
    op->progs.insert(op->progs.end(), bwd.begin(), bwd.end());
    try {
        op_prepare_device(*op);
    } catch (...) {
        delete op;
        throw;
    }
    return op;
}

}  // namespace qs
