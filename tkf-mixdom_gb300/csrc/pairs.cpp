// pairs.cpp -- native reader of the precompiled X/A/Y pair records
// (util/pair_format.py, read by train_pfam.py:984-1029 PrecompiledPairSource).
//
// A shard is JSON lines, one record per line: "x" the ancestor residues and
// "y" the descendant residues as letters of ACDEFGHIKLMNPQRSTVWY (index 0..19
// in that order, util/pair_format.py:23-26), "a" the alignment as a run-length
// string of M/I/D runs ("M5I1M3D2"; a letter followed by a decimal count,
// anything else skipped, util/pair_format.py:68-87), "t" the pair's time,
// "fam" the family; other keys ("id", "gamma", "gamma_lp") are skipped.  The
// reader fills the batch layout of phmm_batch directly -- residues of pair p
// as [x_p, y_p] in one byte array -- and the alignment columns that the 1D
// forward-backward and the match-aligned E-step take: per column its state
// (1 M, 2 I, 3 D), its ancestor character (M, D) and descendant character
// (M, I), 20 where the column has none.  Two passes over the text: a count
// (sizes for the caller's buffers), then the fill.  Records failing the
// consistency rules of validate_record (util/pair_format.py:194-223: M+D runs
// = |x|, M+I runs = |y|, residues in the alphabet) are errors naming the line,
// and so is a line that is not one JSON object (the grammar of numbers,
// literals, strings and escapes is checked; escaped characters are left as
// written, so a residue string with an escape fails the alphabet check).
#include "pairhmm.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <string>

extern "C" __attribute__((visibility("hidden"))) void phmm_internal_set_error(const char *msg);

namespace pf {

// residue letter -> index, 255 outside the alphabet
struct Alphabet {
    unsigned char idx[256];
    Alphabet() {
        std::memset(idx, 255, sizeof idx);
        const char *aa = "ACDEFGHIKLMNPQRSTVWY";
        for (int i = 0; i < 20; ++i) idx[(unsigned char)aa[i]] = (unsigned char)i;
    }
};
static const Alphabet kAlpha;

struct Span {
    const char *p = nullptr;
    size_t n = 0;
};

struct Rec {
    Span x, a, y, fam;
    double t = 0.0;
    bool has_x = false, has_a = false, has_y = false, has_t = false;
};

struct Cur {
    const char *p, *end;
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
    }
};

static bool hexdigit(char ch) {
    return (ch >= '0' && ch <= '9') || (ch >= 'a' && ch <= 'f') || (ch >= 'A' && ch <= 'F');
}

// A JSON string: the raw span between the quotes (escapes checked, left as
// written); control characters and unknown escapes are errors, as in JSON.
static bool str(Cur &c, Span &s) {
    if (c.p >= c.end || *c.p != '"') return false;
    const char *b = ++c.p;
    while (c.p < c.end && *c.p != '"') {
        const unsigned char ch = (unsigned char)*c.p;
        if (ch < 0x20) return false;
        if (ch == '\\') {
            if (c.p + 1 >= c.end) return false;
            const char e = c.p[1];
            if (e == 'u') {
                if (c.end - c.p < 6) return false;
                for (int k = 2; k < 6; ++k)
                    if (!hexdigit(c.p[k])) return false;
                c.p += 6;
                continue;
            }
            if (e == 0 || !std::strchr("\"\\/bfnrt", e)) return false;
            c.p += 2;
            continue;
        }
        ++c.p;
    }
    if (c.p >= c.end) return false;
    s.p = b;
    s.n = (size_t)(c.p - b);
    ++c.p;
    return true;
}

// A JSON number: -?(0|[1-9][0-9]*)(.[0-9]+)?([eE][+-]?[0-9]+)?
static bool number(Cur &c, double &v) {
    const char *b = c.p, *q = c.p;
    auto digits = [&]() {
        const char *d = q;
        while (q < c.end && *q >= '0' && *q <= '9') ++q;
        return q > d;
    };
    if (q < c.end && *q == '-') ++q;
    if (q < c.end && *q == '0') ++q;
    else if (!digits()) return false;
    if (q < c.end && *q == '.') {
        ++q;
        if (!digits()) return false;
    }
    if (q < c.end && (*q == 'e' || *q == 'E')) {
        ++q;
        if (q < c.end && (*q == '+' || *q == '-')) ++q;
        if (!digits()) return false;
    }
    const size_t n = (size_t)(q - b);
    char buf[64];
    if (n >= sizeof buf) return false;
    std::memcpy(buf, b, n);
    buf[n] = 0;
    char *e = nullptr;
    v = std::strtod(buf, &e);
    if (e != buf + n) return false;
    c.p = q;
    return true;
}

// Skip one JSON value of any kind.
static bool skip(Cur &c, int depth = 0) {
    if (depth > 64) return false;
    c.ws();
    if (c.p >= c.end) return false;
    const char ch = *c.p;
    if (ch == '"') {
        Span s;
        return str(c, s);
    }
    if (ch == '[' || ch == '{') {
        const char close = ch == '[' ? ']' : '}';
        ++c.p;
        c.ws();
        if (c.p < c.end && *c.p == close) { ++c.p; return true; }
        for (;;) {
            if (ch == '{') {
                Span k;
                c.ws();
                if (!str(c, k)) return false;
                c.ws();
                if (c.p >= c.end || *c.p != ':') return false;
                ++c.p;
            }
            if (!skip(c, depth + 1)) return false;
            c.ws();
            if (c.p >= c.end) return false;
            if (*c.p == ',') { ++c.p; continue; }
            if (*c.p == close) { ++c.p; return true; }
            return false;
        }
    }
    for (const char *lit : {"true", "false", "null"}) {
        const size_t n = std::strlen(lit);
        if ((size_t)(c.end - c.p) >= n && std::memcmp(c.p, lit, n) == 0) {
            c.p += n;
            return true;
        }
    }
    double v;
    return number(c, v);
}

static bool key_is(const Span &k, const char *name) {
    const size_t n = std::strlen(name);
    return k.n == n && std::memcmp(k.p, name, n) == 0;
}

static bool record(const char *b, const char *e, Rec &r, std::string &err) {
    Cur c{b, e};
    c.ws();
    if (c.p >= c.end || *c.p != '{') { err = "not a JSON object"; return false; }
    ++c.p;
    c.ws();
    if (c.p < c.end && *c.p == '}') { err = "empty record"; return false; }
    for (;;) {
        Span k;
        c.ws();
        if (!str(c, k)) { err = "bad key"; return false; }
        c.ws();
        if (c.p >= c.end || *c.p != ':') { err = "missing ':'"; return false; }
        ++c.p;
        c.ws();
        bool ok;
        if (key_is(k, "x")) ok = r.has_x = str(c, r.x);
        else if (key_is(k, "a")) ok = r.has_a = str(c, r.a);
        else if (key_is(k, "y")) ok = r.has_y = str(c, r.y);
        else if (key_is(k, "fam")) ok = str(c, r.fam);
        else if (key_is(k, "t")) ok = r.has_t = number(c, r.t);
        else ok = skip(c);
        if (!ok) { err = "bad value of key '" + std::string(k.p, k.n) + "'"; return false; }
        c.ws();
        if (c.p < c.end && *c.p == ',') { ++c.p; continue; }
        if (c.p < c.end && *c.p == '}') { ++c.p; break; }
        err = "expected ',' or '}'";
        return false;
    }
    c.ws();
    if (c.p != c.end) { err = "text after the record"; return false; }
    if (!r.has_x || !r.has_a || !r.has_y || !r.has_t) { err = "record needs keys x, a, y and t"; return false; }
    return true;
}

// Run-length alignment: calls f(state, count) per run; returns false on a
// count that does not fit.
template <class Fn>
static bool runs(const Span &a, Fn f) {
    size_t i = 0;
    while (i < a.n) {
        const char ch = a.p[i];
        const int st = ch == 'M' ? 1 : (ch == 'I' ? 2 : (ch == 'D' ? 3 : 0));
        if (st && i + 1 < a.n && a.p[i + 1] >= '0' && a.p[i + 1] <= '9') {
            size_t j = i + 1;
            long long cnt = 0;
            while (j < a.n && a.p[j] >= '0' && a.p[j] <= '9') {
                cnt = cnt * 10 + (a.p[j] - '0');
                if (cnt > (1LL << 30)) return false;
                ++j;
            }
            f(st, cnt);
            i = j;
        } else {
            ++i;
        }
    }
    return true;
}

struct Counts {
    long long m = 0, ins = 0, del = 0;
};

// Shared by both passes: parse line, check it, return its sizes.
static int check(const char *b, const char *e, long long line, Rec &r, Counts &cn) {
    std::string err;
    if (!record(b, e, r, err)) {
        char msg[256];
        snprintf(msg, sizeof msg, "pair records: line %lld: %s", line, err.c_str());
        phmm_internal_set_error(msg);
        return PHMM_E_ARG;
    }
    cn = Counts();
    if (!runs(r.a, [&](int st, long long k) { (st == 1 ? cn.m : (st == 2 ? cn.ins : cn.del)) += k; })) {
        char msg[160];
        snprintf(msg, sizeof msg, "pair records: line %lld: alignment run too long", line);
        phmm_internal_set_error(msg);
        return PHMM_E_ARG;
    }
    char msg[200];
    if (cn.m + cn.del != (long long)r.x.n) {
        snprintf(msg, sizeof msg, "pair records: line %lld: M+D=%lld != len(X)=%zu", line, cn.m + cn.del, r.x.n);
        phmm_internal_set_error(msg);
        return PHMM_E_ARG;
    }
    if (cn.m + cn.ins != (long long)r.y.n) {
        snprintf(msg, sizeof msg, "pair records: line %lld: M+I=%lld != len(Y)=%zu", line, cn.m + cn.ins, r.y.n);
        phmm_internal_set_error(msg);
        return PHMM_E_ARG;
    }
    for (const Span *s : {&r.x, &r.y})
        for (size_t i = 0; i < s->n; ++i)
            if (kAlpha.idx[(unsigned char)s->p[i]] == 255) {
                snprintf(msg, sizeof msg, "pair records: line %lld: invalid residue '%c' in %s", line, s->p[i],
                         s == &r.x ? "X" : "Y");
                phmm_internal_set_error(msg);
                return PHMM_E_ARG;
            }
    return PHMM_OK;
}

template <class Fn>
static int each_line(const char *text, size_t len, Fn f) {
    const char *p = text, *end = text + len;
    long long line = 0;
    while (p < end) {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
        const char *e = nl ? nl : end;
        ++line;
        const char *q = p;
        while (q < e && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q < e) {
            int rc = f(q, e, line);
            if (rc) return rc;
        }
        p = nl ? nl + 1 : end;
    }
    return PHMM_OK;
}

}  // namespace pf

extern "C" int phmm_pairs_count(const char *text, size_t len, phmm_pair_counts *out) {
    using namespace pf;
    if (!out || (!text && len)) {
        phmm_internal_set_error("phmm_pairs_count: null argument");
        return PHMM_E_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    return each_line(text, len, [&](const char *b, const char *e, long long line) {
        Rec r;
        Counts cn;
        int rc = check(b, e, line, r, cn);
        if (rc) return rc;
        out->n_pairs += 1;
        out->n_residues += (int64_t)(r.x.n + r.y.n);
        out->n_columns += cn.m + cn.ins + cn.del;
        return PHMM_OK;
    });
}

extern "C" int phmm_pairs_decode(const char *text, size_t len, const phmm_pair_counts *sizes, int32_t *Lx,
                                 int32_t *Ly, int64_t *x_off, int64_t *y_off, uint8_t *residues, double *t,
                                 int32_t *n_cols, int64_t *col_off, int8_t *col_state, uint8_t *col_anc,
                                 uint8_t *col_desc, int64_t *fam_off, int32_t *fam_len) {
    using namespace pf;
    if (!sizes || (!text && len) ||
        (sizes->n_pairs > 0 && (!Lx || !Ly || !x_off || !y_off || !t || !n_cols || !col_off || !fam_off ||
                                !fam_len)) ||
        (sizes->n_residues > 0 && !residues) ||
        (sizes->n_columns > 0 && (!col_state || !col_anc || !col_desc))) {
        phmm_internal_set_error("phmm_pairs_decode: null argument");
        return PHMM_E_ARG;
    }
    int32_t p = 0;
    int64_t ro = 0, co = 0;
    int rc = each_line(text, len, [&](const char *b, const char *e, long long line) {
        Rec r;
        Counts cn;
        int rc2 = check(b, e, line, r, cn);
        if (rc2) return rc2;
        const int64_t ncol = cn.m + cn.ins + cn.del;
        if (p >= sizes->n_pairs || ro + (int64_t)(r.x.n + r.y.n) > sizes->n_residues || co + ncol > sizes->n_columns) {
            phmm_internal_set_error("phmm_pairs_decode: the text holds more than the counted sizes");
            return PHMM_E_ARG;
        }
        Lx[p] = (int32_t)r.x.n;
        Ly[p] = (int32_t)r.y.n;
        x_off[p] = ro;
        y_off[p] = ro + (int64_t)r.x.n;
        for (size_t i = 0; i < r.x.n; ++i) residues[ro++] = kAlpha.idx[(unsigned char)r.x.p[i]];
        for (size_t i = 0; i < r.y.n; ++i) residues[ro++] = kAlpha.idx[(unsigned char)r.y.p[i]];
        t[p] = r.t;
        n_cols[p] = (int32_t)ncol;
        col_off[p] = co;
        fam_off[p] = r.fam.p ? (int64_t)(r.fam.p - text) : -1;
        fam_len[p] = (int32_t)r.fam.n;
        size_t xi = 0, yj = 0;
        runs(r.a, [&](int st, long long k) {
            for (long long u = 0; u < k; ++u, ++co) {
                col_state[co] = (int8_t)st;
                col_anc[co] = st != 2 ? kAlpha.idx[(unsigned char)r.x.p[xi++]] : 20;
                col_desc[co] = st != 3 ? kAlpha.idx[(unsigned char)r.y.p[yj++]] : 20;
            }
        });
        ++p;
        return PHMM_OK;
    });
    if (rc) return rc;
    if (p != sizes->n_pairs || ro != sizes->n_residues || co != sizes->n_columns) {
        phmm_internal_set_error("phmm_pairs_decode: the text holds less than the counted sizes");
        return PHMM_E_ARG;
    }
    return PHMM_OK;
}
