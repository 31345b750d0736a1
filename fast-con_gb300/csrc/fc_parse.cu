// fc_parse.cu -- edge-list files, parsed by all host threads.
//
// Formats and conventions follow the reference readers:
//   SNAP            load_graph (S/load_graph.c:20-104): '#' comment header,
//                   "# Nodes: N Edges: M", then "u v" per line, raw ids;
//                   readGraphSnap (K/Util/readGraphSTD.cpp:128-145) renumbers
//                   ids by first appearance (relabel = 1).
//   MatrixMarket    "%%MatrixMarket ... [symmetric]", size line, 1-based pairs
//                   (K/Util/readGraphSTD.cpp:57-75).
//   DIMACS9         "p sp N M" and "a u v w" arcs, 1-based
//                   (K/Util/readGraphSTD.cpp:78-99).
//   DIMACS10/METIS  "N M [fmt]" then one line of 1-based neighbours per vertex,
//                   an empty line for a vertex without neighbours
//                   (K/Util/readGraphSTD.cpp:101-125).
// The vertex count is the declared one, raised to max id + 1 if an id
// exceeds it.
//
// The header is read by one thread up to the first edge line; the rest of the
// file is cut at line ends into one chunk per thread.  Each chunk parses into
// its own arrays (DIMACS10 chunks first count their vertex lines so that each
// knows its first vertex id); comment lines met inside the body are kept as
// events and replayed in file order; the chunks are concatenated in file
// order, so the edge order -- and the first-appearance renumbering done
// afterwards -- is that of a sequential read.
#include <algorithm>
#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>

#include "fastcon.h"
#include "fc_internal.cuh"
#include "fc_parse.h"

namespace fc {
namespace {

enum { FMT_NONE = 0, FMT_SNAP = 1, FMT_MM = 2, FMT_D9 = 3, FMT_D10 = 4 };

inline bool is_digit(char c) { return c >= '0' && c <= '9'; }

// parse a (possibly signed) integer at p within [p, e); false if none
inline bool parse_int(const char *&p, const char *e, long long &out)
{
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    if (p >= e) return false;
    bool neg = false;
    if (*p == '-') {
        neg = true;
        ++p;
    }
    if (p >= e || !is_digit(*p)) return false;
    long long v = 0;
    while (p < e && is_digit(*p)) {
        v = v * 10 + (*p - '0');
        if (v > (1ll << 40)) return false;
        ++p;
    }
    out = neg ? -v : v;
    return true;
}

struct Header {
    int fmt = FMT_NONE;
    long long declared = -1;
    int file_directed = -1;
};

// header-type line met in SNAP / MatrixMarket / DIMACS9 text
void header_event(Header &H, const char *line, const char *le)
{
    std::string l(line, le);
    if (H.fmt == FMT_SNAP) {
        if (l.find("Undirected") != std::string::npos)
            H.file_directed = 0;
        else if (l.find("Directed") != std::string::npos && H.file_directed < 0)
            H.file_directed = 1;
        size_t k = l.find("Nodes:");
        if (k != std::string::npos) {
            long long a = -1, b = -1;
            if (sscanf(l.c_str() + k, "Nodes: %lld Edges: %lld", &a, &b) >= 1) H.declared = a;
        }
    } else if (H.fmt == FMT_MM) {
        if (l.compare(0, 14, "%%MatrixMarket") == 0)
            H.file_directed = l.find("symmetric") != std::string::npos ? 0 : 1;
    } else if (H.fmt == FMT_D9) {
        char w1[64], w2[64];
        long long a = -1, b = -1;
        if (sscanf(l.c_str(), "%63s %63s %lld %lld", w1, w2, &a, &b) == 4) H.declared = a;
    }
}

struct Chunk {
    const char *b = nullptr, *e = nullptr;
    std::vector<long long> src, dst;  // raw (SNAP relabel) or final ids
    std::vector<std::pair<const char *, const char *>> events;
    long long maxid = -1;
    long long first_vertex = 0;  // DIMACS10: id of the chunk's first vertex line
    long long vertex_lines = 0;
    int err = 0;
    const char *errmsg = nullptr;
};

inline const char *line_end(const char *p, const char *end)
{
    const char *le = (const char *)memchr(p, '\n', (size_t)(end - p));
    return le ? le : end;
}

// DIMACS10 vertex lines of a chunk: every line but '%' comments
void count_vertex_lines(Chunk &C)
{
    long long n = 0;
    for (const char *p = C.b; p < C.e;) {
        const char *le = line_end(p, C.e);
        const char *q = p;
        while (q < le && (*q == ' ' || *q == '\t')) ++q;
        if (!(q < le && *q == '%')) ++n;
        p = le < C.e ? le + 1 : C.e;
    }
    C.vertex_lines = n;
}

void parse_chunk(Chunk &C, const Header &H, bool keep_raw, long long d10_limit)
{
    auto push = [&](long long a, long long b) -> bool {
        if (a < 0 || b < 0) return false;
        if (!keep_raw && (a > INT_MAX || b > INT_MAX)) return false;
        C.src.push_back(a);
        C.dst.push_back(b);
        C.maxid = std::max(C.maxid, std::max(a, b));
        return true;
    };
    long long vline = C.first_vertex;
    for (const char *p = C.b; p < C.e;) {
        const char *le = line_end(p, C.e);
        const char *q = p;
        while (q < le && (*q == ' ' || *q == '\t')) ++q;
        const char *line = q;
        p = le < C.e ? le + 1 : C.e;
        if (H.fmt == FMT_D10) {
            if (q < le && *q == '%') continue;
            const long long v = vline++;
            if (v >= d10_limit) continue;
            long long a;
            while (parse_int(q, le, a)) {
                if (a < 1 || !push(v, a - 1)) {
                    C.err = FC_ERR_FORMAT;
                    C.errmsg = "malformed METIS adjacency";
                    return;
                }
            }
            continue;
        }
        if (q >= le || *q == '\r') continue;
        long long a, b;
        if (H.fmt == FMT_SNAP) {
            if (*q == '#') {
                C.events.emplace_back(line, le);
                continue;
            }
            if (!parse_int(q, le, a)) continue;
            if (!parse_int(q, le, b) || a < 0 || b < 0) {
                C.err = FC_ERR_FORMAT;
                C.errmsg = "malformed edge line";
                return;
            }
            if (!push(a, b)) {
                C.err = FC_ERR_FORMAT;
                C.errmsg = "vertex id out of range";
                return;
            }
        } else if (H.fmt == FMT_MM) {
            if (*q == '%') {
                C.events.emplace_back(line, le);
                continue;
            }
            if (!parse_int(q, le, a)) continue;
            if (!parse_int(q, le, b) || a < 1 || b < 1 || !push(a - 1, b - 1)) {
                C.err = FC_ERR_FORMAT;
                C.errmsg = "malformed MatrixMarket entry";
                return;
            }
        } else {  // DIMACS9
            if (*q == 'p') {
                C.events.emplace_back(line, le);
                continue;
            }
            if (*q != 'a') continue;
            ++q;
            if (!parse_int(q, le, a) || !parse_int(q, le, b) || a < 1 || b < 1 || !push(a - 1, b - 1)) {
                C.err = FC_ERR_FORMAT;
                C.errmsg = "malformed DIMACS arc";
                return;
            }
        }
    }
}

template <class F>
void run_threads(int n, F f)
{
    if (n <= 1) {
        f(0);
        return;
    }
    std::vector<std::thread> th;
    th.reserve((size_t)n);
    for (int i = 0; i < n; ++i) th.emplace_back(f, i);
    for (auto &t : th) t.join();
}

}  // namespace

int parse_edgelist_file(const char *path, int relabel, int nthreads, Parsed &P)
{
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error("cannot open %s: %s", path, strerror(errno));
        return FC_ERR_IO;
    }
    std::string buf;
    if (fseek(f, 0, SEEK_END) == 0) {
        long sz = ftell(f);
        if (sz > 0) {
            buf.resize((size_t)sz);
            fseek(f, 0, SEEK_SET);
            if (fread(&buf[0], 1, (size_t)sz, f) != (size_t)sz) {
                fclose(f);
                set_error("cannot read %s", path);
                return FC_ERR_IO;
            }
        }
    }
    fclose(f);
    const char *p = buf.data(), *end = buf.data() + buf.size();

    // ---- header, one thread: up to the first line that may carry an edge
    Header H;
    bool mm_size = false, d10_header = false;
    const char *body = end;
    while (p < end) {
        const char *le = line_end(p, end);
        const char *q = p;
        while (q < le && (*q == ' ' || *q == '\t')) ++q;
        const char *line = q;
        const char *next = le < end ? le + 1 : end;
        if (q >= le || *q == '\r') {
            p = next;
            continue;
        }
        if (H.fmt == FMT_NONE) {
            if (*q == '#')
                H.fmt = FMT_SNAP;
            else if (le - q >= 14 && memcmp(q, "%%MatrixMarket", 14) == 0)
                H.fmt = FMT_MM;
            else if (*q == 'c' || *q == 'p')
                H.fmt = FMT_D9;
            else if (*q == '%' || is_digit(*q))
                H.fmt = FMT_D10;
            else {
                set_error("%s: unrecognised graph format", path);
                return FC_ERR_FORMAT;
            }
        }
        if (H.fmt == FMT_SNAP) {
            if (*q != '#') {
                body = p;
                break;
            }
            header_event(H, line, le);
        } else if (H.fmt == FMT_MM) {
            if (*q == '%') {
                header_event(H, line, le);
            } else if (!mm_size) {
                long long a, b, c;
                if (parse_int(q, le, a)) {
                    if (!parse_int(q, le, b) || !parse_int(q, le, c)) {
                        set_error("%s: malformed MatrixMarket size line", path);
                        return FC_ERR_FORMAT;
                    }
                    H.declared = a;
                    mm_size = true;
                }
            } else {
                body = p;
                break;
            }
        } else if (H.fmt == FMT_D9) {
            if (*q == 'a') {
                body = p;
                break;
            }
            if (*q == 'p') header_event(H, line, le);
        } else {  // DIMACS10: '%' comments, then "N M [fmt]"
            if (*q != '%') {
                long long a, b, c;
                if (parse_int(q, le, a)) {
                    if (!parse_int(q, le, b)) {
                        set_error("%s: malformed METIS header", path);
                        return FC_ERR_FORMAT;
                    }
                    H.declared = a;
                    H.file_directed = (parse_int(q, le, c) && c == 100) ? 1 : 0;
                    d10_header = true;
                    body = next;
                    break;
                }
            }
        }
        p = next;
    }
    if (H.fmt == FMT_NONE) {
        set_error("%s: empty file", path);
        return FC_ERR_FORMAT;
    }
    (void)d10_header;

    // ---- body, all threads
    int T = nthreads > 0 ? nthreads : (int)std::thread::hardware_concurrency();
    if (T < 1) T = 1;
    const size_t bytes = (size_t)(end - body);
    T = (int)std::min<size_t>((size_t)std::min(T, 64), bytes / (1 << 20) + 1);
    std::vector<Chunk> ch((size_t)T);
    const char *cur = body;
    for (int i = 0; i < T; ++i) {
        const char *e = i + 1 == T ? end : body + bytes * (size_t)(i + 1) / (size_t)T;
        if (e < cur) e = cur;
        if (e < end) {
            const char *nl = (const char *)memchr(e, '\n', (size_t)(end - e));
            e = nl ? nl + 1 : end;
        }
        ch[(size_t)i].b = cur;
        ch[(size_t)i].e = e;
        cur = e;
    }
    const bool keep_raw = relabel && H.fmt == FMT_SNAP;
    long long d10_limit = LLONG_MAX;
    if (H.fmt == FMT_D10) {
        run_threads(T, [&](int i) { count_vertex_lines(ch[(size_t)i]); });
        long long first = 0;
        for (auto &C : ch) {
            C.first_vertex = first;
            first += C.vertex_lines;
        }
        d10_limit = H.declared;
    }
    run_threads(T, [&](int i) { parse_chunk(ch[(size_t)i], H, keep_raw, d10_limit); });

    // ---- merge in file order
    size_t total = 0;
    long long maxid = -1;
    for (auto &C : ch) {
        if (C.err) {
            set_error("%s: %s", path, C.errmsg);
            return C.err;
        }
        for (auto &ev : C.events) header_event(H, ev.first, ev.second);
        total += C.src.size();
        maxid = std::max(maxid, C.maxid);
    }
    P.src.resize(total);
    P.dst.resize(total);
    long long nv = H.declared;
    if (keep_raw) {
        // first-appearance renumbering in file order: a then b of each line
        std::unordered_map<long long, int32_t> idmap;
        idmap.reserve(total / 4 + 16);
        size_t k = 0;
        for (auto &C : ch)
            for (size_t j = 0; j < C.src.size(); ++j, ++k) {
                auto ia = idmap.emplace(C.src[j], (int32_t)idmap.size()).first;
                P.src[k] = ia->second;
                auto ib = idmap.emplace(C.dst[j], (int32_t)idmap.size()).first;
                P.dst[k] = ib->second;
            }
        // the header's node count when it is larger (vertices that appear
        // in no edge), as readGraphHeader sizes the graph from it
        maxid = (long long)idmap.size() - 1;
        nv = std::max((long long)idmap.size(), H.declared);
    } else {
        std::vector<size_t> off(ch.size() + 1, 0);
        for (size_t i = 0; i < ch.size(); ++i) off[i + 1] = off[i] + ch[i].src.size();
        run_threads(T, [&](int i) {
            const Chunk &C = ch[(size_t)i];
            for (size_t j = 0; j < C.src.size(); ++j) {
                P.src[off[(size_t)i] + j] = (int32_t)C.src[j];
                P.dst[off[(size_t)i] + j] = (int32_t)C.dst[j];
            }
        });
    }
    P.file_directed = H.file_directed;
    if (nv < maxid + 1) nv = maxid + 1;
    if (nv > INT_MAX) {
        set_error("%s: %lld vertices exceed the int32 limit", path, nv);
        return FC_ERR_OVERFLOW;
    }
    P.nv = nv;
    return FC_OK;
}

}  // namespace fc
