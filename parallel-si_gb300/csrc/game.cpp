// game.cpp -- host-side parity game: CSR arrays, the pgsolver .gm reader and
// writer, and the seeded generators.
//
// The reader follows the reference's Game::parse_pgsolver (game.cpp:51-107):
// the first line is discarded, empty lines are skipped, each vertex line is
// `id priority owner s1,s2,... [label];`, ids must run 0,1,2,... in order, and
// the messages of the reference's exceptions are kept.  Two inputs the reference
// accepts but then indexes out of bounds with are rejected here: negative
// priorities and successor ids outside [0, n).  Files ending in .gz are read
// through zlib when the library was built with it (the reference uses boost
// iostreams for .gz and .bz2, main.cpp:140-151; .bz2 is not supported).
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <climits>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#ifdef PSI_HAVE_ZLIB
#include <zlib.h>
#endif

#include "game.h"
#include "psi_internal.h"

namespace psi {

namespace {

struct Cursor {
    const char *p, *end;
    bool eol() const { return p >= end; }
    void skip_ws()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) p++;
    }
    // operator>>(int&) semantics: optional sign then digits; false on no digits
    // or overflow.
    bool read_int(int32_t &out)
    {
        skip_ws();
        const char *q = p;
        bool neg = false;
        if (q < end && (*q == '+' || *q == '-')) {
            neg = (*q == '-');
            q++;
        }
        if (q >= end || *q < '0' || *q > '9') return false;
        int64_t v = 0;
        while (q < end && *q >= '0' && *q <= '9') {
            v = v * 10 + (*q - '0');
            if (v > (int64_t)INT32_MAX + 1) return false;
            q++;
        }
        if (neg) v = -v;
        if (v > INT32_MAX || v < INT32_MIN) return false;
        out = (int32_t)v;
        p = q;
        return true;
    }
    bool read_char(char &c)
    {
        skip_ws();
        if (p >= end) return false;
        c = *p++;
        return true;
    }
};

int parse_error(const std::string &what, int64_t line_no)
{
    return fail(PSI_ERR_PARSE, "parsing error: " + what + " (line " + std::to_string(line_no) + ")");
}

}  // namespace

int parse_gm(const char *text, int64_t len, HostGame &g)
{
    g = HostGame();
    g.offsets.assign(1, 0);
    if (len <= 0) return PSI_OK;                    // no header line: empty game (game.cpp:56)
    const char *p = text, *end = text + len;
    int64_t line_no = 0;
    // discard the header line (game.cpp:56)
    const char *nl = (const char *)memchr(p, '\n', end - p);
    p = nl ? nl + 1 : end;
    line_no = 1;
    IVec offsets;
    offsets.push_back(0);
    while (p < end) {
        nl = (const char *)memchr(p, '\n', end - p);
        const char *le = nl ? nl : end;
        line_no++;
        Cursor c{p, le};
        p = nl ? nl + 1 : end;
        c.skip_ws();
        if (c.eol()) continue;                          // empty line
        // id: leading integer of the first token (stoi semantics)
        const char *tok = c.p;
        while (c.p < c.end && !(*c.p == ' ' || *c.p == '\t' || *c.p == '\r' || *c.p == '\v' || *c.p == '\f')) c.p++;
        Cursor tc{tok, c.p};
        int32_t id;
        if (!tc.read_int(id)) return parse_error("invalid id token", line_no);
        if (id < 0) return parse_error("invalid id", line_no);
        int32_t pri, owner;
        if (!c.read_int(pri)) return parse_error("missing priority", line_no);
        if (!c.read_int(owner)) return parse_error("missing player", line_no);
        if (owner != 0 && owner != 1) return parse_error("invalid player", line_no);
        if (id != (int32_t)g.owner.size())
            return parse_error("vertices must be listed in order starting at 0!", line_no);
        if (pri < 0) return parse_error("negative priority", line_no);
        g.owner.push_back(owner);
        g.priority.push_back(pri);
        int64_t deg = 0;
        for (;;) {
            int32_t to;
            if (!c.read_int(to)) return parse_error("missing successor", line_no);
            g.targets.push_back(to);
            deg++;
            char ch;
            if (!c.read_char(ch)) return parse_error("missing ; to end line", line_no);
            if (ch != ',') break;
        }
        if (deg == 0) return parse_error("sinks are not allowed!", line_no);
        if ((int64_t)g.targets.size() > INT32_MAX) return fail(PSI_ERR_TOO_LARGE, "more than 2^31-1 edges");
        offsets.push_back((int32_t)g.targets.size());
    }
    g.n = (int32_t)g.owner.size();
    g.m = (int64_t)g.targets.size();
    g.offsets.swap(offsets);
    int32_t mp = 0;
    for (int32_t v = 0; v < g.n; v++) mp = g.priority[v] > mp ? g.priority[v] : mp;
    g.max_pri = mp;
    for (int64_t e = 0; e < g.m; e++)
        if (g.targets[e] < 0 || g.targets[e] >= g.n)
            return fail(PSI_ERR_PARSE, "parsing error: successor " + std::to_string(g.targets[e]) +
                                           " out of range");
    return PSI_OK;
}

int load_gm(const char *path, HostGame &g)
{
    std::string s(path ? path : "");
    std::vector<char> buf;
    bool gz = s.size() > 3 && s.compare(s.size() - 3, 3, ".gz") == 0;
    bool bz = s.size() > 4 && s.compare(s.size() - 4, 4, ".bz2") == 0;
    if (bz) return fail(PSI_ERR_IO, "bzip2-compressed games are not supported: " + s);
    if (gz) {
#ifdef PSI_HAVE_ZLIB
        gzFile f = gzopen(s.c_str(), "rb");
        if (!f) return fail(PSI_ERR_IO, "Unable to open file: " + s);
        char chunk[1 << 16];
        int r;
        while ((r = gzread(f, chunk, sizeof chunk)) > 0) buf.insert(buf.end(), chunk, chunk + r);
        int errnum = 0;
        if (r < 0) {
            gzerror(f, &errnum);
            gzclose(f);
            return fail(PSI_ERR_IO, "gzip read error: " + s);
        }
        gzclose(f);
#else
        return fail(PSI_ERR_IO, "this build has no zlib: cannot read " + s);
#endif
    } else {
        FILE *f = fopen(s.c_str(), "rb");
        if (!f) return fail(PSI_ERR_IO, "Unable to open file: " + s);
        fseek(f, 0, SEEK_END);
        long sz = ftell(f);
        fseek(f, 0, SEEK_SET);
        buf.resize(sz > 0 ? (size_t)sz : 0);
        if (sz > 0 && fread(buf.data(), 1, (size_t)sz, f) != (size_t)sz) {
            fclose(f);
            return fail(PSI_ERR_IO, "read error: " + s);
        }
        fclose(f);
    }
    return parse_gm(buf.data(), (int64_t)buf.size(), g);
}

int write_gm(const HostGame &g, const char *path)
{
    FILE *f = fopen(path, "wb");
    if (!f) return fail(PSI_ERR_IO, std::string("cannot write ") + path);
    std::vector<char> out;
    out.reserve(1 << 20);
    char tmp[64];
    auto put = [&](const char *s, int k) { out.insert(out.end(), s, s + k); };
    int k = snprintf(tmp, sizeof tmp, "parity %d;\n", g.n - 1);
    put(tmp, k);
    for (int32_t v = 0; v < g.n; v++) {
        k = snprintf(tmp, sizeof tmp, "%d %d %d ", v, g.priority[v], g.owner[v]);
        put(tmp, k);
        for (int32_t e = g.offsets[v]; e < g.offsets[v + 1]; e++) {
            k = snprintf(tmp, sizeof tmp, e + 1 < g.offsets[v + 1] ? "%d," : "%d;\n", g.targets[e]);
            put(tmp, k);
        }
        if (out.size() > (1u << 24)) {
            fwrite(out.data(), 1, out.size(), f);
            out.clear();
        }
    }
    fwrite(out.data(), 1, out.size(), f);
    bool ok = (fclose(f) == 0);
    return ok ? PSI_OK : fail(PSI_ERR_IO, std::string("write error: ") + path);
}

void parallel_chunks(int64_t count, const std::function<void(int64_t, int64_t)> &f)
{
    int64_t threads = (int64_t)std::thread::hardware_concurrency();
    threads = std::max<int64_t>(1, std::min<int64_t>(threads, 16));
    threads = std::min<int64_t>(threads, count / (1 << 20) + 1);
    if (threads <= 1) {
        if (count > 0) f(0, count);
        return;
    }
    std::vector<std::thread> pool;
    for (int64_t t = 0; t < threads; t++) {
        int64_t lo = count * t / threads, hi = count * (t + 1) / threads;
        pool.emplace_back([&f, lo, hi] { f(lo, hi); });
    }
    for (auto &th : pool) th.join();
}

namespace {

// First failing vertex check (in vertex order) over [lo, hi): 1 bad player,
// 2 negative priority, 3 no successor; returns (vertex, kind) or (-1, 0).
std::pair<int64_t, int> first_bad_vertex(int64_t lo, int64_t hi, const int32_t *owner, const int32_t *priority,
                                         const int32_t *offsets)
{
    for (int64_t v = lo; v < hi; v++) {
        if (owner[v] != 0 && owner[v] != 1) return {v, 1};
        if (priority[v] < 0) return {v, 2};
        if (offsets[v + 1] <= offsets[v]) return {v, 3};
    }
    return {-1, 0};
}

}  // namespace

int validate_csr(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
                 const int32_t *targets)
{
    if (n < 0) return fail(PSI_ERR_INVALID, "negative vertex count");
    if (offsets[0] != 0) return fail(PSI_ERR_INVALID, "offsets[0] must be 0");
    if (n == 0) return PSI_OK;   // the empty game (offsets = {0})
    // vertex checks per chunk; the lowest failing vertex decides the message
    std::mutex mu;
    std::pair<int64_t, int> worst{-1, 0};
    parallel_chunks(n, [&](int64_t lo, int64_t hi) {
        auto b = first_bad_vertex(lo, hi, owner, priority, offsets);
        if (b.first < 0) return;
        std::lock_guard<std::mutex> lk(mu);
        if (worst.first < 0 || b.first < worst.first) worst = b;
    });
    if (worst.first >= 0) {
        std::string v = std::to_string(worst.first);
        if (worst.second == 1) return fail(PSI_ERR_INVALID, "invalid player at vertex " + v);
        if (worst.second == 2) return fail(PSI_ERR_INVALID, "negative priority at vertex " + v);
        return fail(PSI_ERR_INVALID, "vertex " + v + " has no successor");
    }
    std::atomic<bool> bad_edge{false};
    parallel_chunks(offsets[n], [&](int64_t lo, int64_t hi) {
        for (int64_t e = lo; e < hi; e++)
            if (targets[e] < 0 || targets[e] >= n) {
                bad_edge = true;
                return;
            }
    });
    if (bad_edge) return fail(PSI_ERR_INVALID, "successor out of range");
    return PSI_OK;
}

namespace {

int32_t max_priority(int32_t n, const int32_t *priority)
{
    std::mutex mu;
    int32_t mp = 0;
    parallel_chunks(n, [&](int64_t lo, int64_t hi) {
        int32_t local = 0;
        for (int64_t v = lo; v < hi; v++) local = priority[v] > local ? priority[v] : local;
        std::lock_guard<std::mutex> lk(mu);
        mp = local > mp ? local : mp;
    });
    return mp;
}

}  // namespace

int make_view(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
              const int32_t *targets, CsrView &v)
{
    int rc = validate_csr(n, owner, priority, offsets, targets);
    if (rc) return rc;
    v = CsrView{n, offsets[n], max_priority(n, priority), owner, priority, offsets, targets};
    return PSI_OK;
}

// Validation is read-only and runs on several threads; the copy stays on one
// (first-touch page faults from many threads were slower than one copy).
int make_game(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
              const int32_t *targets, HostGame &g)
{
    CsrView v;
    int rc = make_view(n, owner, priority, offsets, targets, v);
    if (rc) return rc;
    g.n = n;
    g.m = v.m;
    g.max_pri = v.max_pri;
    g.owner.resize(n);
    g.priority.resize(n);
    g.offsets.resize((size_t)n + 1);
    g.targets.resize(g.m);
    std::memcpy(g.owner.data(), owner, 4 * (size_t)n);
    std::memcpy(g.priority.data(), priority, 4 * (size_t)n);
    std::memcpy(g.offsets.data(), offsets, 4 * ((size_t)n + 1));
    std::memcpy(g.targets.data(), targets, 4 * (size_t)g.m);
    return PSI_OK;
}

int generate_random(int32_t n, int32_t deg_lo, int32_t deg_hi, int32_t pri_hi, uint64_t seed, HostGame &g)
{
    g = HostGame();
    g.offsets.resize((size_t)n + 1);
    int rc = gen_random_offsets(n, deg_lo, deg_hi, seed, g.offsets.data());
    if (rc) return fail(rc, "invalid random-game parameters");
    g.n = n;
    g.m = g.offsets[n];
    g.owner.resize(n);
    g.priority.resize(n);
    g.targets.resize(g.m);
    rc = gen_random_fill(n, deg_lo, deg_hi, pri_hi, seed, g.offsets.data(), g.owner.data(), g.priority.data(),
                         g.targets.data());
    if (rc) return fail(rc, "invalid random-game parameters");
    int32_t mp = 0;
    for (int32_t v = 0; v < n; v++) mp = g.priority[v] > mp ? g.priority[v] : mp;
    g.max_pri = mp;
    return PSI_OK;
}

int generate_longpath(int32_t n, int32_t pri_hi, uint64_t seed, HostGame &g)
{
    g = HostGame();
    if (n < 2 || pri_hi < 1) return fail(PSI_ERR_INVALID, "invalid long-path parameters");
    g.offsets.resize((size_t)n + 1);
    g.owner.resize(n);
    g.priority.resize(n);
    g.targets.resize(2 * (size_t)n);
    int rc = gen_longpath(n, pri_hi, seed, g.owner.data(), g.priority.data(), g.offsets.data(), g.targets.data());
    if (rc) return fail(rc, "invalid long-path parameters");
    g.n = n;
    g.m = g.offsets[n];
    g.targets.resize(g.m);
    int32_t mp = 0;
    for (int32_t v = 0; v < n; v++) mp = g.priority[v] > mp ? g.priority[v] : mp;
    g.max_pri = mp;
    return PSI_OK;
}

}  // namespace psi
