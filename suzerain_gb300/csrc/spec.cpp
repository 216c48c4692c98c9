// Solver specification strings ("zgbsv", "zgbsvx,equil=true",
// "zcgbsvx,reuse=false,aiter=5,siter=25,diter=5,tolsc=145"): parse and
// format with the grammar and defaults of suzerain::specification_zgbsv
// (suzerain/specification_zgbsv.cpp:46-158), written as a small
// recursive-descent parser: keywords are case-insensitive, whitespace may
// appear between any two tokens, the zcgbsvx options may come in any order
// but each at most once, and the whole string must be consumed.
#include "suzerain_gb300.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

namespace {

struct Cursor {
    const char *p, *end;
    void ws() { while (p < end && std::isspace((unsigned char) *p)) ++p; }
    // case-insensitive keyword (after whitespace); advances on success
    bool kw(const char *w)
    {
        ws();
        const char *q = p;
        for (; *w; ++w, ++q)
            if (q >= end || std::tolower((unsigned char) *q) != *w) return false;
        p = q;
        return true;
    }
    bool ch(char c)
    {
        ws();
        if (p < end && *p == c) { ++p; return true; }
        return false;
    }
    bool boolean(int *out)
    {
        if (kw("true")) { *out = 1; return true; }
        if (kw("false")) { *out = 0; return true; }
        return false;
    }
    bool integer(int *out)
    {
        ws();
        const char *q = p;
        bool neg = false;
        if (q < end && (*q == '+' || *q == '-')) neg = (*q++ == '-');
        if (q >= end || !std::isdigit((unsigned char) *q)) return false;
        long long v = 0;
        while (q < end && std::isdigit((unsigned char) *q)) {
            v = v * 10 + (*q++ - '0');
            if (v > 2147483648ll) return false;
        }
        if (neg) v = -v;
        if (v > 2147483647ll || v < -2147483648ll) return false;
        *out = (int) v;
        p = q;
        return true;
    }
    // [+-]? ( digits [ . digits* ] | . digits ) ( [eE] [+-]? digits )?  |  nan | inf | infinity
    bool real(double *out)
    {
        ws();
        const char *q = p;
        bool neg = false;
        if (q < end && (*q == '+' || *q == '-')) neg = (*q++ == '-');
        Cursor c{q, end};
        if (c.kw("nan")) { *out = std::nan(""); p = c.p; return true; }
        if (c.kw("infinity") || c.kw("inf")) { *out = neg ? -INFINITY : INFINITY; p = c.p; return true; }
        const char *s = q;
        int digits = 0;
        while (q < end && std::isdigit((unsigned char) *q)) { ++q; ++digits; }
        if (q < end && *q == '.') {
            ++q;
            while (q < end && std::isdigit((unsigned char) *q)) { ++q; ++digits; }
        }
        if (!digits) return false;
        if (q < end && (*q == 'e' || *q == 'E')) {
            const char *r = q + 1;
            if (r < end && (*r == '+' || *r == '-')) ++r;
            if (r < end && std::isdigit((unsigned char) *r)) {
                while (r < end && std::isdigit((unsigned char) *r)) ++r;
                q = r;
            }
        }
        const std::string num(s, q);
        const double v = std::strtod(num.c_str(), nullptr);
        *out = neg ? -v : v;
        p = q;
        return true;
    }
};

void set_err(char *err, size_t len, const char *spec, const char *at)
{
    if (err && len) std::snprintf(err, len, "spec_zgbsv specification '%s' invalid beginning with '%s'",
                                  spec, at);
}

}  // namespace

extern "C" void sgb_solver_spec_default(sgb_solver_spec *s)
{
    if (!s) return;
    s->method = SGB_METHOD_ZCGBSVX;
    s->equil = 0;
    s->reuse = 0;
    s->aiter = 1;
    s->siter = -1;
    s->diter = 5;
    s->tolsc = 0.0;
}

extern "C" int sgb_solver_spec_parse(const char *spec, sgb_solver_spec *out, char *err,
                                     size_t errlen)
{
    if (!spec || !out) return -1;
    sgb_solver_spec s;
    sgb_solver_spec_default(&s);
    Cursor c{spec, spec + std::strlen(spec)};
    c.ws();
    if (c.p != c.end) {
        bool ok = false;
        Cursor save = c;
        if (c.kw("zgbsvx")) {
            s.method = SGB_METHOD_ZGBSVX;
            ok = true;
            Cursor opt = c;
            int b;
            if (opt.ch(',') && opt.kw("equil") && opt.ch('=') && opt.boolean(&b)) {
                s.equil = b;
                c = opt;
            }
        } else if ((c = save, c.kw("zgbsv"))) {
            s.method = SGB_METHOD_ZGBSV;
            ok = true;
        } else if ((c = save, c.kw("zcgbsvx"))) {
            s.method = SGB_METHOD_ZCGBSVX;
            ok = true;
            bool seen[5] = {false, false, false, false, false};
            for (;;) {
                Cursor opt = c;
                if (!opt.ch(',')) break;
                int iv, b;
                double dv;
                if (!seen[0] && opt.kw("reuse") && opt.ch('=') && opt.boolean(&b)) {
                    s.reuse = b; seen[0] = true;
                } else if ((opt = c, opt.ch(',')) && !seen[1] && opt.kw("aiter") && opt.ch('=') && opt.integer(&iv)) {
                    s.aiter = iv; seen[1] = true;
                } else if ((opt = c, opt.ch(',')) && !seen[2] && opt.kw("siter") && opt.ch('=') && opt.integer(&iv)) {
                    s.siter = iv; seen[2] = true;
                } else if ((opt = c, opt.ch(',')) && !seen[3] && opt.kw("diter") && opt.ch('=') && opt.integer(&iv)) {
                    s.diter = iv; seen[3] = true;
                } else if ((opt = c, opt.ch(',')) && !seen[4] && opt.kw("tolsc") && opt.ch('=') && opt.real(&dv)) {
                    s.tolsc = dv; seen[4] = true;
                } else {
                    break;
                }
                c = opt;
            }
        } else {
            c = save;
        }
        c.ws();
        if (!ok || c.p != c.end) {
            set_err(err, errlen, spec, c.p);
            return -1;
        }
    }
    *out = s;
    return 0;
}

extern "C" int sgb_solver_spec_format(const sgb_solver_spec *s, char *buf, size_t len)
{
    if (!s || !buf || !len) return -1;
    int n;
    switch (s->method) {
    case SGB_METHOD_ZGBSV:
        n = std::snprintf(buf, len, "zgbsv");
        break;
    case SGB_METHOD_ZGBSVX:
        n = std::snprintf(buf, len, "zgbsvx,equil=%s", s->equil ? "true" : "false");
        break;
    case SGB_METHOD_ZCGBSVX:
        n = std::snprintf(buf, len, "zcgbsvx,reuse=%s,aiter=%d,siter=%d,diter=%d,tolsc=%g",
                          s->reuse ? "true" : "false", s->aiter, s->siter, s->diter, s->tolsc);
        break;
    default:
        n = std::snprintf(buf, len, "UNKNOWN");
    }
    return (n < 0 || (size_t) n >= len) ? -1 : 0;
}
