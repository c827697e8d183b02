// host_graph.cpp -- edge-list loading and synthetic graph generation (host side).
//
// Loader: same rules as Graph::ReadGraph (reference src/graph.cpp:12-113):
//   * dispatch on the file extension: .edges .el .wel .txt .edgelist are text, .bcsr .bwcsr binary;
//   * a text line whose first character is not a digit is skipped (comments, blank lines,
//     lines starting with whitespace) -- src/graph.cpp:66-67;
//   * the first two whitespace-separated unsigned integers are source and end; the third, when it
//     parses, is the weight, else the weight is 1 (src/graph.cpp:87-93); anything after is ignored;
//   * num_nodes = the largest id seen, +1 when an id 0 occurs (src/graph.cpp:102-105).
//   Tokens follow `istream >> unsigned` (optional sign, digits, stops at the first non-digit; a
//   missing end id reads as 0, a missing or malformed weight as 1; a value above UINT_MAX reads as
//   UINT_MAX). The file is memory-mapped and parsed by several threads over line-aligned chunks;
//   the result is identical to a single-threaded parse.
// Binary: Subway's CSR files (Subway/tools/converter.cpp:90-93, 159-162): u32 num_nodes, u32 num_edges,
//   u32 nodePointer[num_nodes], then u32 end (.bcsr) or {u32 end, u32 w8} (.bwcsr) per edge. The
//   reference's own reader reads these records as {source,end} pairs and never fills the weights
//   (src/graph.cpp:19-34); this reader decodes the format as Subway writes it.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

#include "internal.hpp"

namespace {

std::string file_extension(const std::string& path) {
    const size_t dot = path.find_last_of('.');
    return dot == std::string::npos ? std::string() : path.substr(dot + 1);
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }
inline bool is_digit(char c) { return c >= '0' && c <= '9'; }

// Parse one unsigned token at p (within [p, e)); returns false on failure (value set per the
// istream rules described above). Advances p.
inline bool parse_u32(const char*& p, const char* e, uint32_t& out) {
    while (p < e && is_space(*p)) ++p;
    bool neg = false;
    const char* q = p;
    if (q < e && (*q == '+' || *q == '-')) {
        neg = (*q == '-');
        ++q;
    }
    if (q >= e || !is_digit(*q)) {
        out = 0;
        return false;
    }
    uint64_t v = 0;
    bool over = false;
    while (q < e && is_digit(*q)) {
        if (!over) {
            v = v * 10u + (uint64_t)(*q - '0');
            if (v > 0xFFFFFFFFull) over = true;
        }
        ++q;
    }
    p = q;
    if (over) {
        out = 0xFFFFFFFFu;
        return false;
    }
    out = neg ? (uint32_t)(0u - (uint32_t)v) : (uint32_t)v;
    return true;
}

struct Chunk {
    std::vector<uint32_t> s, d, w;
    uint32_t max = 0;
    bool zero = false;
};

void parse_chunk(const char* b, const char* e, bool weighted, Chunk& c) {
    const char* p = b;
    while (p < e) {
        const char* nl = (const char*)memchr(p, '\n', (size_t)(e - p));
        const char* le = nl ? nl : e;
        if (le > p && is_digit(*p)) {
            const char* q = p;
            uint32_t s = 0, d = 0, w = 1;
            bool ok = parse_u32(q, le, s);
            if (ok) ok = parse_u32(q, le, d);
            else d = 0;
            if (weighted) {
                uint32_t tw = 1;
                if (ok && parse_u32(q, le, tw)) w = tw;
                else w = 1;
            }
            c.s.push_back(s);
            c.d.push_back(d);
            if (weighted) c.w.push_back(w);
            if (s == 0 || d == 0) c.zero = true;
            c.max = std::max(c.max, std::max(s, d));
        }
        p = nl ? nl + 1 : e;
    }
}

eeg_status load_text(const std::string& path, bool weighted, int n_threads, eeg_graph* g) {
    int fd = open(path.c_str(), O_RDONLY);
    if (fd < 0) {
        eeg::set_last_error("cannot open " + path);
        return EEG_ERR_IO;
    }
    struct stat st;
    if (fstat(fd, &st) != 0) {
        close(fd);
        eeg::set_last_error("cannot stat " + path);
        return EEG_ERR_IO;
    }
    const size_t size = (size_t)st.st_size;
    const char* data = nullptr;
    void* map = nullptr;
    if (size > 0) {
        map = mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
        if (map == MAP_FAILED) {
            close(fd);
            eeg::set_last_error("cannot map " + path);
            return EEG_ERR_IO;
        }
        data = (const char*)map;
    }
    int T = n_threads > 0 ? n_threads : (int)std::max(1u, std::thread::hardware_concurrency());
    if (size < (1u << 20)) T = 1;
    std::vector<const char*> cuts(T + 1);
    cuts[0] = data;
    cuts[T] = data + size;
    for (int i = 1; i < T; ++i) {
        const char* c = data + size * (size_t)i / (size_t)T;
        if (c < cuts[i - 1]) c = cuts[i - 1];
        const char* nl = (const char*)memchr(c, '\n', (size_t)(data + size - c));
        cuts[i] = nl ? nl + 1 : data + size;
    }
    std::vector<Chunk> chunks(T);
    std::vector<std::thread> th;
    for (int i = 0; i < T; ++i)
        th.emplace_back([&, i] { parse_chunk(cuts[i], std::max(cuts[i], cuts[i + 1]), weighted, chunks[i]); });
    for (auto& t : th) t.join();
    if (map) munmap(map, size);
    close(fd);
    size_t m = 0;
    uint32_t mx = 0;
    bool zero = false;
    for (auto& c : chunks) {
        m += c.s.size();
        mx = std::max(mx, c.max);
        zero = zero || c.zero;
    }
    g->src.reserve(m);
    g->dst.reserve(m);
    if (weighted) g->weight.reserve(m);
    for (auto& c : chunks) {
        g->src.insert(g->src.end(), c.s.begin(), c.s.end());
        g->dst.insert(g->dst.end(), c.d.begin(), c.d.end());
        if (weighted) g->weight.insert(g->weight.end(), c.w.begin(), c.w.end());
    }
    g->num_edges = m;
    g->has_zero_id = zero;
    g->num_nodes = zero ? mx + 1u : mx;
    g->is_weighted = weighted;
    return EEG_OK;
}

eeg_status load_bcsr(const std::string& path, bool weighted_file, bool want_weights, eeg_graph* g) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        eeg::set_last_error("cannot open " + path);
        return EEG_ERR_IO;
    }
    uint32_t n = 0, m = 0;
    f.read((char*)&n, 4);
    f.read((char*)&m, 4);
    if (!f) {
        eeg::set_last_error("truncated header in " + path);
        return EEG_ERR_IO;
    }
    std::vector<uint32_t> np(n);
    f.read((char*)np.data(), (std::streamsize)n * 4);
    std::vector<uint32_t> rec((size_t)m * (weighted_file ? 2 : 1));
    f.read((char*)rec.data(), (std::streamsize)rec.size() * 4);
    if (!f) {
        eeg::set_last_error("truncated body in " + path);
        return EEG_ERR_IO;
    }
    g->src.resize(m);
    g->dst.resize(m);
    if (want_weights) g->weight.assign(m, 1u);
    for (uint32_t v = 0; v < n; ++v) {
        const uint32_t a = np[v], b = (v + 1 < n) ? np[v + 1] : m;
        if (a > b || b > m) {
            eeg::set_last_error("corrupt node pointers in " + path);
            return EEG_ERR_IO;
        }
        for (uint32_t e = a; e < b; ++e) {
            g->src[e] = v;
            g->dst[e] = weighted_file ? rec[2 * (size_t)e] : rec[e];
            if (want_weights && weighted_file) g->weight[e] = rec[2 * (size_t)e + 1];
        }
    }
    for (uint32_t e = 0; e < m; ++e)
        if (g->dst[e] >= n) {
            eeg::set_last_error("edge target outside num_nodes in " + path);
            return EEG_ERR_IO;
        }
    g->num_nodes = n;
    g->num_edges = m;
    g->has_zero_id = true;  // CSR ids are 0-based by construction
    g->is_weighted = want_weights;
    return EEG_OK;
}

// ------------------------------------------------------------------ counter-based RNG
inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t hash2(uint64_t a, uint64_t b) { return mix64(a ^ mix64(b + 0x632BE59BD9B4E019ull)); }

template <class F>
void parallel_for(uint64_t n, F f) {
    const unsigned T = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 64u));
    if (n < 65536 || T == 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    for (unsigned i = 0; i < T; ++i) {
        const uint64_t a = n * i / T, b = n * (i + 1) / T;
        th.emplace_back([=] { f(a, b); });
    }
    for (auto& t : th) t.join();
}

}  // namespace

extern "C" {

EEG_API eeg_status eeg_graph_load(const char* path, int weighted, int n_threads, eeg_graph** out) {
    if (!path || !out) {
        eeg::set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    *out = nullptr;
    const std::string p(path), ext = file_extension(p);
    eeg_graph* g = new eeg_graph();
    eeg_status s;
    if (ext == "bcsr" || ext == "bwcsr") s = load_bcsr(p, ext == "bwcsr", weighted != 0, g);
    else if (ext == "edges" || ext == "el" || ext == "wel" || ext == "txt" || ext == "edgelist")
        s = load_text(p, weighted != 0, n_threads, g);
    else {
        eeg::set_last_error("Graph file type not recognized: " + p);
        s = EEG_ERR_IO;
    }
    if (s != EEG_OK) {
        delete g;
        return s;
    }
    *out = g;
    return EEG_OK;
}

EEG_API eeg_status eeg_graph_from_arrays(uint32_t num_nodes, uint64_t num_edges, const uint32_t* src,
                                         const uint32_t* dst, const uint32_t* weight, eeg_graph** out) {
    if (!out || (num_edges && (!src || !dst))) {
        eeg::set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    eeg_graph* g = new eeg_graph();
    g->num_nodes = num_nodes;
    g->num_edges = num_edges;
    g->has_zero_id = true;
    g->is_weighted = true;
    g->src.assign(src, src + num_edges);
    g->dst.assign(dst, dst + num_edges);
    if (weight) g->weight.assign(weight, weight + num_edges);
    else g->weight.assign(num_edges, 1u);
    *out = g;
    return EEG_OK;
}

EEG_API eeg_status eeg_graph_view_get(const eeg_graph* g, eeg_graph_view* v) {
    if (!g || !v) {
        eeg::set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    v->num_nodes = g->num_nodes;
    v->num_edges = g->num_edges;
    v->has_zero_id = g->has_zero_id;
    v->is_weighted = g->is_weighted;
    v->src = g->src.data();
    v->dst = g->dst.data();
    v->weight = g->weight.empty() ? nullptr : g->weight.data();
    return EEG_OK;
}

EEG_API eeg_status eeg_graph_normalized_ids(const eeg_graph* g, uint32_t* s, uint32_t* d) {
    if (!g) {
        eeg::set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    const uint32_t shift = g->has_zero_id ? 0u : 1u;
    for (uint64_t e = 0; e < g->num_edges; ++e) {
        if (s) s[e] = g->src[e] - shift;
        if (d) d[e] = g->dst[e] - shift;
    }
    return EEG_OK;
}

EEG_API void eeg_graph_destroy(eeg_graph* g) { delete g; }

EEG_API eeg_status eeg_graph_save_bcsr(const eeg_graph* g, const char* path) {
    if (!g || !path) {
        eeg::set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    const std::string ext = file_extension(path);
    const bool weighted = ext == "bwcsr";
    if (!weighted && ext != "bcsr") {
        eeg::set_last_error("extension must be .bcsr or .bwcsr");
        return EEG_ERR_INVALID;
    }
    if (g->num_edges > 0xFFFFFFFFull) {
        eeg::set_last_error("too many edges for the 32-bit CSR format");
        return EEG_ERR_INVALID;
    }
    const uint32_t shift = g->has_zero_id ? 0u : 1u;
    const uint32_t n = g->num_nodes;
    const uint32_t m = (uint32_t)g->num_edges;
    std::vector<uint32_t> deg(n + 1, 0), pos;
    for (uint64_t e = 0; e < m; ++e) {
        const uint32_t s = g->src[e] - shift;
        if (s >= n || g->dst[e] - shift >= n) {
            eeg::set_last_error("edge endpoint outside num_nodes");
            return EEG_ERR_INVALID;
        }
        deg[s]++;
    }
    std::vector<uint32_t> np(n);
    uint32_t acc = 0;
    for (uint32_t v = 0; v < n; ++v) {
        np[v] = acc;
        acc += deg[v];
    }
    pos = np;
    std::vector<uint32_t> rec((size_t)m * (weighted ? 2 : 1));
    for (uint64_t e = 0; e < m; ++e) {  // stable: input order within a vertex
        const uint32_t s = g->src[e] - shift;
        const uint32_t at = pos[s]++;
        if (weighted) {
            rec[2 * (size_t)at] = g->dst[e] - shift;
            rec[2 * (size_t)at + 1] = g->weight.empty() ? 1u : g->weight[e];
        } else {
            rec[at] = g->dst[e] - shift;
        }
    }
    std::ofstream f(path, std::ios::binary);
    if (!f) {
        eeg::set_last_error(std::string("cannot write ") + path);
        return EEG_ERR_IO;
    }
    f.write((const char*)&n, 4);
    f.write((const char*)&m, 4);
    f.write((const char*)np.data(), (std::streamsize)n * 4);
    f.write((const char*)rec.data(), (std::streamsize)rec.size() * 4);
    return f ? EEG_OK : EEG_ERR_IO;
}

EEG_API eeg_status eeg_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                                uint32_t wmin, uint32_t wmax, uint32_t* src, uint32_t* dst, uint32_t* weight) {
    if (!src || !dst || scale == 0 || scale > 31 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0 ||
        (weight && wmax < wmin)) {
        eeg::set_last_error("invalid R-MAT parameters");
        return EEG_ERR_INVALID;
    }
    const uint64_t m = (uint64_t)edge_factor << scale;
    const double two32 = 4294967296.0;
    const uint64_t tA = (uint64_t)std::floor(a * two32);
    const uint64_t tAB = (uint64_t)std::floor((a + b) * two32);
    const uint64_t tABC = (uint64_t)std::floor((a + b + c) * two32);
    const uint64_t range = (uint64_t)wmax - wmin + 1u;
    parallel_for(m, [=](uint64_t lo, uint64_t hi) {
        for (uint64_t e = lo; e < hi; ++e) {
            const uint64_t s0 = hash2(seed, e);
            uint32_t u = 0, v = 0;
            uint64_t r = 0;
            for (uint32_t l = 0; l < scale; ++l) {
                if ((l & 1u) == 0) r = mix64(s0 + 0x9E3779B97F4A7C15ull * (l / 2 + 1));
                const uint64_t x = (l & 1u) ? (r >> 32) : (r & 0xFFFFFFFFull);
                const uint32_t bit = 1u << (scale - 1 - l);
                if (x < tA) {
                } else if (x < tAB) {
                    v |= bit;
                } else if (x < tABC) {
                    u |= bit;
                } else {
                    u |= bit;
                    v |= bit;
                }
            }
            src[e] = u;
            dst[e] = v;
            if (weight) weight[e] = wmin + (uint32_t)(mix64(s0 ^ 0xA5A5A5A55A5A5A5Aull) % range);
        }
    });
    return EEG_OK;
}

EEG_API eeg_status eeg_gen_grid(uint32_t side, double p_delete, double shortcut_frac, uint64_t seed, uint32_t wmin,
                                uint32_t wmax, uint64_t* num_arcs, uint32_t* src, uint32_t* dst, uint32_t* weight) {
    if (!num_arcs || side < 2 || (uint64_t)side * side > 0xFFFFFFFFull || p_delete < 0 || p_delete > 1 ||
        shortcut_frac < 0 || wmax < wmin) {
        eeg::set_last_error("invalid grid parameters");
        return EEG_ERR_INVALID;
    }
    const uint64_t S = side, N = S * S;
    const uint64_t E = 2 * S * (S - 1);  // undirected grid edges
    const uint64_t nshort = (uint64_t)std::llround(shortcut_frac * (double)E);
    const uint64_t thr = p_delete >= 1.0 ? ~0ull : (uint64_t)(p_delete * 18446744073709551616.0);
    const uint64_t range = (uint64_t)wmax - wmin + 1u;
    auto kept = [=](uint64_t i) { return p_delete <= 0 || mix64(hash2(seed, i)) >= thr; };
    auto endpoints = [=](uint64_t i, uint32_t& u, uint32_t& v) {
        if (i < S * (S - 1)) {  // horizontal (r,c)-(r,c+1)
            const uint64_t r = i / (S - 1), c = i % (S - 1);
            u = (uint32_t)(r * S + c);
            v = (uint32_t)(r * S + c + 1);
        } else if (i < E) {     // vertical (r,c)-(r+1,c)
            const uint64_t j = i - S * (S - 1);
            const uint64_t r = j / S, c = j % S;
            u = (uint32_t)(r * S + c);
            v = (uint32_t)((r + 1) * S + c);
        } else {                // shortcut
            const uint64_t j = i - E;
            u = (uint32_t)(hash2(seed ^ 0x5CA1AB1Eull, 2 * j) % N);
            v = (uint32_t)(hash2(seed ^ 0x5CA1AB1Eull, 2 * j + 1) % N);
        }
    };
    const uint64_t total = E + nshort;
    // count kept undirected edges per block, then write at block offsets (deterministic)
    const uint64_t B = 1u << 16;
    const uint64_t nb = (total + B - 1) / B;
    std::vector<uint64_t> cnt(nb + 1, 0);
    parallel_for(nb, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t b = lo; b < hi; ++b) {
            uint64_t c = 0;
            for (uint64_t i = b * B; i < std::min(total, (b + 1) * B); ++i) c += (i >= E || kept(i)) ? 1 : 0;
            cnt[b + 1] = c;
        }
    });
    for (uint64_t b = 0; b < nb; ++b) cnt[b + 1] += cnt[b];
    *num_arcs = 2 * cnt[nb];
    if (!src) return EEG_OK;
    if (!dst) {
        eeg::set_last_error("null dst");
        return EEG_ERR_INVALID;
    }
    parallel_for(nb, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t b = lo; b < hi; ++b) {
            uint64_t o = 2 * cnt[b];
            for (uint64_t i = b * B; i < std::min(total, (b + 1) * B); ++i) {
                if (!(i >= E || kept(i))) continue;
                uint32_t u, v;
                endpoints(i, u, v);
                const uint32_t w = wmin + (uint32_t)(hash2(seed ^ 0x77EE77EEull, i) % range);
                src[o] = u; dst[o] = v;
                src[o + 1] = v; dst[o + 1] = u;
                if (weight) weight[o] = weight[o + 1] = w;
                o += 2;
            }
        }
    });
    return EEG_OK;
}

EEG_API eeg_status eeg_symmetrize(uint64_t m, const uint32_t* src, const uint32_t* dst, const uint32_t* w,
                                  uint32_t* so, uint32_t* d_o, uint32_t* wo) {
    if ((m && (!src || !dst || !so || !d_o)) || (wo && !w && m)) {
        eeg::set_last_error("null argument");
        return EEG_ERR_INVALID;
    }
    parallel_for(m, [=](uint64_t lo, uint64_t hi) {
        for (uint64_t e = lo; e < hi; ++e) {
            so[e] = src[e];
            d_o[e] = dst[e];
            so[m + e] = dst[e];
            d_o[m + e] = src[e];
            if (wo) wo[e] = wo[m + e] = w[e];
        }
    });
    return EEG_OK;
}

}  // extern "C"
