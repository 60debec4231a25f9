// Synthetic graph generators and CSR assembly (host, OpenMP).
//
// The reference reads its inputs from files (bfs/src/biio.h:21-149) and, for
// undirected use, merges a CSR with its transpose (bfs/src/main.c:130-169,
// bfs/src/utils.c:351-379). Here the same end state -- a symmetric CSR with
// ascending, duplicate-free rows -- is produced from generated edge lists.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "albba_gen.h"
#include "internal.h"

#ifdef _OPENMP
#include <omp.h>
#endif

using alb::fail;
using alb::mix64;
using alb::u01;

namespace {

constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

// Independent streams per purpose so that e.g. the permutation does not
// correlate with edge draws.
enum Stream : uint64_t {
    kEdges = 0x52A7E1ull,
    kPerm = 0x9E4A11ull,
    kDrop = 0xD409ull,
    kShortcut = 0x5C0417ull,
    kRoots = 0x4007ull,
};

inline uint64_t stream_base(uint64_t seed, Stream s) { return mix64(mix64(seed) ^ (uint64_t)s); }
inline uint64_t draw(uint64_t base, uint64_t ctr) { return mix64(base + ctr * kGamma); }

template <class T>
T *xmalloc(size_t count) {
    T *p = (T *)std::malloc(sizeof(T) * (count ? count : 1));
    if (!p) throw std::bad_alloc();
    return p;
}

// Exclusive scan of a[0..n) into a[0..n], a[n] = total.
void exclusive_scan_inplace(int64_t *a, int64_t n) {
    int64_t acc = 0;
    for (int64_t i = 0; i < n; i++) {
        int64_t t = a[i];
        a[i] = acc;
        acc += t;
    }
    a[n] = acc;
}

alb_status csr_from_edges(int64_t n, int64_t m, const int32_t *u, const int32_t *v,
                          alb_host_csr *out) {
    std::vector<int64_t> cnt((size_t)n + 1, 0);
    int bad = 0;
#pragma omp parallel for reduction(| : bad)
    for (int64_t e = 0; e < m; e++) {
        int32_t a = u[e], b = v[e];
        if (a < 0 || b < 0 || a >= n || b >= n) {
            bad |= 1;
            continue;
        }
        if (a == b) continue;
        __atomic_fetch_add(&cnt[a], 1, __ATOMIC_RELAXED);
        __atomic_fetch_add(&cnt[b], 1, __ATOMIC_RELAXED);
    }
    if (bad) return fail(ALB_ERR_INVALID, "edge endpoint outside [0, %lld)", (long long)n);
    exclusive_scan_inplace(cnt.data(), n);
    int64_t total = cnt[n];
    int32_t *tmp = xmalloc<int32_t>((size_t)total);
    std::vector<int64_t> cur(cnt.begin(), cnt.end());
#pragma omp parallel for
    for (int64_t e = 0; e < m; e++) {
        int32_t a = u[e], b = v[e];
        if (a == b) continue;
        tmp[__atomic_fetch_add(&cur[a], 1, __ATOMIC_RELAXED)] = b;
        tmp[__atomic_fetch_add(&cur[b], 1, __ATOMIC_RELAXED)] = a;
    }
    std::vector<int64_t> uniq((size_t)n + 1, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t r = 0; r < n; r++) {
        int32_t *lo = tmp + cnt[r], *hi = tmp + cnt[r + 1];
        std::sort(lo, hi);
        uniq[r] = std::unique(lo, hi) - lo;
    }
    exclusive_scan_inplace(uniq.data(), n);
    out->n = n;
    out->nnz = uniq[n];
    out->rowptr = xmalloc<int64_t>((size_t)n + 1);
    out->col = xmalloc<int32_t>((size_t)uniq[n]);
    std::memcpy(out->rowptr, uniq.data(), sizeof(int64_t) * ((size_t)n + 1));
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < n; r++)
        std::memcpy(out->col + uniq[r], tmp + cnt[r], sizeof(int32_t) * (size_t)(uniq[r + 1] - uniq[r]));
    std::free(tmp);
    return ALB_OK;
}

template <class F>
alb_status guarded(F &&f) {
    try {
        return f();
    } catch (const std::bad_alloc &) {
        return fail(ALB_ERR_OOM, "host allocation failed");
    }
}

}  // namespace

extern "C" {

alb_status alb_csr_from_edges(int64_t n, int64_t m, const int32_t *u, const int32_t *v,
                              alb_host_csr *out) {
    if (!out || n <= 0 || n > INT32_MAX || m < 0 || (m > 0 && (!u || !v)))
        return fail(ALB_ERR_INVALID, "alb_csr_from_edges: bad arguments");
    std::memset(out, 0, sizeof(*out));
    return guarded([&] { return csr_from_edges(n, m, u, v, out); });
}

alb_status alb_gen_rmat(int32_t scale, int32_t edgefactor, uint64_t seed, double a, double b,
                        double c, int32_t permute, alb_host_csr *out) {
    if (!out || scale < 1 || scale > 30 || edgefactor < 1 || a < 0 || b < 0 || c < 0 ||
        a + b + c > 1.0)
        return fail(ALB_ERR_INVALID, "alb_gen_rmat: bad arguments");
    std::memset(out, 0, sizeof(*out));
    return guarded([&]() -> alb_status {
        const int64_t n = int64_t(1) << scale;
        const int64_t m = (int64_t)edgefactor * n;
        int32_t *eu = xmalloc<int32_t>((size_t)m), *ev = xmalloc<int32_t>((size_t)m);
        const uint64_t be = stream_base(seed, kEdges);
        const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < m; e++) {
            uint32_t x = 0, y = 0;
            for (int32_t l = 0; l < scale; l++) {
                double r = u01(draw(be, (uint64_t)e * (uint64_t)scale + (uint64_t)l));
                uint32_t bx = (r >= ab) ? 1u : 0u;             // quadrants C, D: row bit
                uint32_t by = (r >= a && r < ab) || r >= abc;  // quadrants B, D: col bit
                x = (x << 1) | bx;
                y = (y << 1) | by;
            }
            eu[e] = (int32_t)x;
            ev[e] = (int32_t)y;
        }
        if (permute) {
            int32_t *perm = xmalloc<int32_t>((size_t)n);
            for (int64_t i = 0; i < n; i++) perm[i] = (int32_t)i;
            const uint64_t bp = stream_base(seed, kPerm);
            for (int64_t i = n - 1; i > 0; i--) {  // Fisher-Yates
                int64_t j = (int64_t)(draw(bp, (uint64_t)i) % (uint64_t)(i + 1));
                std::swap(perm[i], perm[j]);
            }
#pragma omp parallel for schedule(static)
            for (int64_t e = 0; e < m; e++) {
                eu[e] = perm[eu[e]];
                ev[e] = perm[ev[e]];
            }
            std::free(perm);
        }
        alb_status st = csr_from_edges(n, m, eu, ev, out);
        std::free(eu);
        std::free(ev);
        return st;
    });
}

alb_status alb_gen_grid(int32_t rows, int32_t cols, double drop, double shortcut_frac,
                        uint64_t seed, alb_host_csr *out) {
    if (!out || rows < 1 || cols < 1 || (int64_t)rows * cols > INT32_MAX || drop < 0 ||
        drop > 1 || shortcut_frac < 0)
        return fail(ALB_ERR_INVALID, "alb_gen_grid: bad arguments");
    std::memset(out, 0, sizeof(*out));
    return guarded([&]() -> alb_status {
        const int64_t n = (int64_t)rows * cols;
        const int64_t nh = (int64_t)rows * (cols - 1), nv = (int64_t)(rows - 1) * cols;
        const int64_t ns = (int64_t)(shortcut_frac * (double)n + 0.5);
        const int64_t cap = nh + nv + ns;
        int32_t *eu = xmalloc<int32_t>((size_t)cap), *ev = xmalloc<int32_t>((size_t)cap);
        const uint64_t bd = stream_base(seed, kDrop), bs = stream_base(seed, kShortcut);
        // Dropped grid edges become self-loops, which CSR assembly discards.
#pragma omp parallel for schedule(static)
        for (int64_t id = 0; id < nh + nv; id++) {
            int64_t a, b;
            if (id < nh) {
                int64_t r = id / (cols - 1), c = id % (cols - 1);
                a = r * cols + c;
                b = a + 1;
            } else {
                int64_t k = id - nh;
                a = k;
                b = k + cols;
            }
            bool keep = u01(draw(bd, (uint64_t)id)) >= drop;
            eu[id] = (int32_t)a;
            ev[id] = (int32_t)(keep ? b : a);
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < ns; i++) {
            eu[nh + nv + i] = (int32_t)(draw(bs, 2 * (uint64_t)i) % (uint64_t)n);
            ev[nh + nv + i] = (int32_t)(draw(bs, 2 * (uint64_t)i + 1) % (uint64_t)n);
        }
        alb_status st = csr_from_edges(n, cap, eu, ev, out);
        std::free(eu);
        std::free(ev);
        return st;
    });
}

alb_status alb_gen_er(int64_t n, double mean_degree, uint64_t seed, alb_host_csr *out) {
    if (!out || n < 1 || n > INT32_MAX || mean_degree < 0)
        return fail(ALB_ERR_INVALID, "alb_gen_er: bad arguments");
    std::memset(out, 0, sizeof(*out));
    return guarded([&]() -> alb_status {
        const int64_t m = (int64_t)((double)n * mean_degree / 2.0 + 0.5);
        int32_t *eu = xmalloc<int32_t>((size_t)m), *ev = xmalloc<int32_t>((size_t)m);
        const uint64_t be = stream_base(seed, kEdges);
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < m; e++) {
            eu[e] = (int32_t)(draw(be, 2 * (uint64_t)e) % (uint64_t)n);
            ev[e] = (int32_t)(draw(be, 2 * (uint64_t)e + 1) % (uint64_t)n);
        }
        alb_status st = csr_from_edges(n, m, eu, ev, out);
        std::free(eu);
        std::free(ev);
        return st;
    });
}

alb_status alb_pick_roots(const alb_host_csr *g, int32_t count, uint64_t seed, int32_t *roots) {
    if (!g || !g->rowptr || !roots || count < 0)
        return fail(ALB_ERR_INVALID, "alb_pick_roots: bad arguments");
    const uint64_t br = stream_base(seed, kRoots);
    int32_t got = 0;
    const uint64_t max_tries = (uint64_t)count * 64 + (uint64_t)4 * (uint64_t)g->n + 1024;
    for (uint64_t t = 0; t < max_tries && got < count; t++) {
        int32_t v = (int32_t)(draw(br, t) % (uint64_t)g->n);
        if (g->rowptr[v + 1] == g->rowptr[v]) continue;
        bool dup = false;
        for (int32_t i = 0; i < got; i++) dup |= roots[i] == v;
        if (!dup) roots[got++] = v;
    }
    if (got < count)
        return fail(ALB_ERR_INVALID, "alb_pick_roots: only %d vertices with degree >= 1", got);
    return ALB_OK;
}

void alb_host_csr_free(alb_host_csr *g) {
    if (!g) return;
    std::free(g->rowptr);
    std::free(g->col);
    g->rowptr = nullptr;
    g->col = nullptr;
    g->n = g->nnz = 0;
}

alb_status alb_cbd_write(const char *path, const alb_host_csr *g) {
    if (!path || !g || !g->rowptr || g->n > INT32_MAX || g->nnz > INT32_MAX)
        return fail(ALB_ERR_INVALID, "alb_cbd_write: bad arguments or graph too large for int32");
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return fail(ALB_ERR_IO, "alb_cbd_write: cannot open %s", path);
    int32_t hdr[3] = {(int32_t)g->n, (int32_t)g->n, (int32_t)g->nnz};
    bool ok = std::fwrite(hdr, sizeof(int32_t), 3, fp) == 3;
    std::vector<int32_t> rp((size_t)g->n + 1);
    for (int64_t i = 0; i <= g->n; i++) rp[i] = (int32_t)g->rowptr[i];
    ok = ok && std::fwrite(rp.data(), sizeof(int32_t), rp.size(), fp) == rp.size();
    ok = ok && std::fwrite(g->col, sizeof(int32_t), (size_t)g->nnz, fp) == (size_t)g->nnz;
    std::vector<double> ones(1 << 16, 1.0);
    for (int64_t done = 0; ok && done < g->nnz;) {
        size_t k = (size_t)std::min<int64_t>((int64_t)ones.size(), g->nnz - done);
        ok = std::fwrite(ones.data(), sizeof(double), k, fp) == k;
        done += (int64_t)k;
    }
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? ALB_OK : fail(ALB_ERR_IO, "alb_cbd_write: short write to %s", path);
}

alb_status alb_cbd_read(const char *path, alb_host_csr *out) {
    if (!path || !out) return fail(ALB_ERR_INVALID, "alb_cbd_read: bad arguments");
    std::memset(out, 0, sizeof(*out));
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return fail(ALB_ERR_IO, "alb_cbd_read: cannot open %s", path);
    return guarded([&]() -> alb_status {
        int32_t hdr[3];
        if (std::fread(hdr, sizeof(int32_t), 3, fp) != 3 || hdr[0] < 0 || hdr[2] < 0 ||
            hdr[0] != hdr[1]) {
            std::fclose(fp);
            return fail(ALB_ERR_IO, "alb_cbd_read: bad header in %s", path);
        }
        const int64_t n = hdr[0], nnz = hdr[2];
        std::vector<int32_t> rp((size_t)n + 1);
        int32_t *col = xmalloc<int32_t>((size_t)nnz);
        bool ok = std::fread(rp.data(), sizeof(int32_t), rp.size(), fp) == rp.size() &&
                  std::fread(col, sizeof(int32_t), (size_t)nnz, fp) == (size_t)nnz;
        // values are ignored (forced to 1.0 by the reference, main.c:106-109),
        // but must be present for the file to be complete.
        std::vector<double> vbuf(1 << 16);
        for (int64_t done = 0; ok && done < nnz;) {
            size_t k = (size_t)std::min<int64_t>((int64_t)vbuf.size(), nnz - done);
            ok = std::fread(vbuf.data(), sizeof(double), k, fp) == k;
            done += (int64_t)k;
        }
        std::fclose(fp);
        ok = ok && rp[0] == 0 && rp[n] == nnz;
        for (int64_t i = 0; ok && i < n; i++) ok = rp[i] <= rp[i + 1];
        for (int64_t e = 0; ok && e < nnz; e++) ok = col[e] >= 0 && col[e] < n;
        if (!ok) {
            std::free(col);
            return fail(ALB_ERR_IO, "alb_cbd_read: truncated or inconsistent file %s", path);
        }
        out->n = n;
        out->nnz = nnz;
        out->rowptr = xmalloc<int64_t>((size_t)n + 1);
        for (int64_t i = 0; i <= n; i++) out->rowptr[i] = rp[i];
        out->col = col;
        return ALB_OK;
    });
}


}  // extern "C"

// ------------------------------------------------------------ Matrix Market
// Reader of coordinate Matrix Market files with the reference's semantics
// (bfs/src/mmio_highlevel.h:140-263, banner rules of mmio.h:248-330): the
// banner's type (real, integer, complex, pattern) only decides how many
// numbers follow the two 1-based indices, and values are dropped (the
// reference overwrites them with 1.0, main.c:106-109); a symmetric or
// hermitian file stores each off-diagonal entry once and the CSR receives it
// in both rows; entries go into their rows in file order, the mirrored copy
// at its source entry's turn. Skew-symmetric files are read as general, as
// the reference does. Dense (array) files, non-square matrices and indices
// out of range are refused, where the reference would misread them.
namespace {

struct MtxFile {
    FILE *fp = nullptr;
    ~MtxFile() {
        if (fp) std::fclose(fp);
    }
};

bool next_data_line(FILE *fp, std::vector<char> &buf) {
    for (;;) {
        if (!std::fgets(buf.data(), (int)buf.size(), fp)) return false;
        const char *c = buf.data();
        while (*c == ' ' || *c == '\t') c++;
        if (*c == '%' || *c == '\n' || *c == '\r' || *c == '\0') continue;  // comment, blank
        return true;
    }
}

std::string lower(const char *s) {
    std::string r(s);
    for (char &ch : r) ch = (char)std::tolower((unsigned char)ch);
    return r;
}

}  // namespace

extern "C" {

alb_status alb_mtx_read(const char *path, alb_host_csr *out, int32_t *is_symmetric) {
    if (!path || !out) return fail(ALB_ERR_INVALID, "alb_mtx_read: bad arguments");
    std::memset(out, 0, sizeof(*out));
    if (is_symmetric) *is_symmetric = 0;
    MtxFile f;
    f.fp = std::fopen(path, "r");
    if (!f.fp) return fail(ALB_ERR_IO, "alb_mtx_read: cannot open %s", path);
    return guarded([&]() -> alb_status {
        std::vector<char> line(1 << 16);
        if (!std::fgets(line.data(), (int)line.size(), f.fp))
            return fail(ALB_ERR_IO, "alb_mtx_read: %s is empty", path);
        char banner[64] = {0}, obj[64] = {0}, fmt[64] = {0}, type[64] = {0}, sym[64] = {0};
        if (std::sscanf(line.data(), "%63s %63s %63s %63s %63s", banner, obj, fmt, type, sym) != 5 ||
            std::strncmp(banner, "%%MatrixMarket", 14) != 0 || lower(obj) != "matrix")
            return fail(ALB_ERR_IO, "alb_mtx_read: %s has no Matrix Market banner", path);
        const std::string sf = lower(fmt), st = lower(type), ss = lower(sym);
        if (sf == "array")
            return fail(ALB_ERR_UNSUPPORTED, "alb_mtx_read: %s is a dense (array) file", path);
        int extra;  // numbers after the two indices
        if (st == "pattern") extra = 0;
        else if (st == "real" || st == "integer") extra = 1;
        else if (st == "complex") extra = 2;
        else return fail(ALB_ERR_IO, "alb_mtx_read: %s: unknown type %s", path, type);
        bool mirror;
        if (ss == "symmetric" || ss == "hermitian") mirror = true;
        else if (ss == "general" || ss == "skew-symmetric") mirror = false;
        else return fail(ALB_ERR_IO, "alb_mtx_read: %s: unknown symmetry %s", path, sym);
        if (sf != "coordinate")
            return fail(ALB_ERR_IO, "alb_mtx_read: %s: unknown format %s", path, fmt);
        long long rows = 0, cols = 0, entries = 0;
        if (!next_data_line(f.fp, line) ||
            std::sscanf(line.data(), "%lld %lld %lld", &rows, &cols, &entries) != 3 || rows < 0 ||
            cols < 0 || entries < 0)
            return fail(ALB_ERR_IO, "alb_mtx_read: %s: bad size line", path);
        if (rows != cols)
            return fail(ALB_ERR_UNSUPPORTED, "alb_mtx_read: %s is %lld x %lld, not square", path,
                        rows, cols);
        if (rows > INT32_MAX)
            return fail(ALB_ERR_UNSUPPORTED, "alb_mtx_read: %s: %lld rows exceed int32 ids", path,
                        rows);
        const int64_t n = rows;
        std::vector<int32_t> ei((size_t)entries), ej((size_t)entries);
        for (long long e = 0; e < entries; e++) {
            if (!next_data_line(f.fp, line))
                return fail(ALB_ERR_IO, "alb_mtx_read: %s ends after %lld of %lld entries", path, e,
                            entries);
            char *c = line.data(), *end = nullptr;
            const long long i = std::strtoll(c, &end, 10);
            if (end == c) return fail(ALB_ERR_IO, "alb_mtx_read: %s: bad entry %lld", path, e + 1);
            c = end;
            const long long j = std::strtoll(c, &end, 10);
            if (end == c) return fail(ALB_ERR_IO, "alb_mtx_read: %s: bad entry %lld", path, e + 1);
            c = end;
            for (int k = 0; k < extra; k++) {  // the value(s): checked, then dropped
                std::strtod(c, &end);
                if (end == c)
                    return fail(ALB_ERR_IO, "alb_mtx_read: %s: entry %lld lacks its value", path,
                                e + 1);
                c = end;
            }
            if (i < 1 || i > rows || j < 1 || j > cols)
                return fail(ALB_ERR_IO, "alb_mtx_read: %s: entry %lld (%lld, %lld) outside %lld x %lld",
                            path, e + 1, i, j, rows, cols);
            ei[(size_t)e] = (int32_t)(i - 1);
            ej[(size_t)e] = (int32_t)(j - 1);
        }
        // rows counted, then filled in file order (the mirrored copy at its
        // source entry's turn)
        std::vector<int64_t> cnt((size_t)n + 1, 0);
        for (long long e = 0; e < entries; e++) {
            cnt[(size_t)ei[(size_t)e]]++;
            if (mirror && ei[(size_t)e] != ej[(size_t)e]) cnt[(size_t)ej[(size_t)e]]++;
        }
        exclusive_scan_inplace(cnt.data(), n);
        const int64_t nnz = cnt[(size_t)n];
        int64_t *rp = xmalloc<int64_t>((size_t)n + 1);
        int32_t *col = xmalloc<int32_t>((size_t)nnz);
        std::memcpy(rp, cnt.data(), sizeof(int64_t) * ((size_t)n + 1));
        std::vector<int64_t> at(cnt.begin(), cnt.end() - 1);
        for (long long e = 0; e < entries; e++) {
            const int32_t i = ei[(size_t)e], j = ej[(size_t)e];
            col[at[(size_t)i]++] = j;
            if (mirror && i != j) col[at[(size_t)j]++] = i;
        }
        out->n = n;
        out->nnz = nnz;
        out->rowptr = rp;
        out->col = col;
        if (is_symmetric) *is_symmetric = mirror ? 1 : 0;
        return ALB_OK;
    });
}

// The reference driver's conversion of a non-symmetric graph to an
// undirected one (bfs/src/main.c:127-163): row i of the result merges row i
// of the transpose (ascending: the transpose is filled row by row of the
// input) with row i of the input by the two-pointer merge of
// bfs/src/utils.c:351-380, which emits an element once when both heads are
// equal. On ascending rows that is the sorted union; on unsorted input rows
// the result keeps the reference's order and repeats.
alb_status alb_csr_undirected(const alb_host_csr *in, alb_host_csr *out) {
    if (!in || !out || in->n < 0 || (in->n > 0 && (!in->rowptr || (in->nnz > 0 && !in->col))))
        return fail(ALB_ERR_INVALID, "alb_csr_undirected: bad arguments");
    std::memset(out, 0, sizeof(*out));
    return guarded([&]() -> alb_status {
        const int64_t n = in->n, nnz = in->nnz;
        if (in->rowptr[0] != 0 || in->rowptr[n] != nnz)
            return fail(ALB_ERR_INVALID, "alb_csr_undirected: row offsets do not span the entries");
        for (int64_t i = 0; i < n; i++)
            if (in->rowptr[i] > in->rowptr[i + 1])
                return fail(ALB_ERR_INVALID, "alb_csr_undirected: row offsets decrease at %lld",
                            (long long)i);
        for (int64_t e = 0; e < nnz; e++)
            if (in->col[e] < 0 || in->col[e] >= n)
                return fail(ALB_ERR_INVALID, "alb_csr_undirected: column outside [0, %lld)",
                            (long long)n);
        // transpose: tp / trow, rows of the transpose ascending
        std::vector<int64_t> tp((size_t)n + 1, 0);
        for (int64_t e = 0; e < nnz; e++) tp[(size_t)in->col[e]]++;
        exclusive_scan_inplace(tp.data(), n);
        std::vector<int32_t> trow((size_t)nnz);
        {
            std::vector<int64_t> at(tp.begin(), tp.end() - 1);
            for (int64_t i = 0; i < n; i++)
                for (int64_t e = in->rowptr[i]; e < in->rowptr[i + 1]; e++)
                    trow[(size_t)at[(size_t)in->col[e]]++] = (int32_t)i;
        }
        int64_t *rp = xmalloc<int64_t>((size_t)n + 1);
        int32_t *col = xmalloc<int32_t>((size_t)(2 * nnz));
        int64_t len = 0;
        for (int64_t i = 0; i < n; i++) {
            const int32_t *a = trow.data() + tp[(size_t)i], *b = in->col + in->rowptr[i];
            const int64_t al = tp[(size_t)i + 1] - tp[(size_t)i], bl = in->rowptr[i + 1] - in->rowptr[i];
            int64_t x = 0, y = 0;
            rp[i] = len;
            while (x < al && y < bl) {
                if (a[x] < b[y]) col[len++] = a[x++];
                else if (a[x] == b[y]) {
                    col[len++] = b[y++];
                    x++;
                } else col[len++] = b[y++];
            }
            while (x < al) col[len++] = a[x++];
            while (y < bl) col[len++] = b[y++];
        }
        rp[n] = len;
        out->n = n;
        out->nnz = len;
        out->rowptr = rp;
        out->col = col;
        return ALB_OK;
    });
}

// Graph load as the reference driver does it (bfs/src/main.c:86-163,
// biio.h:127-149): .cbd read as is; .mtx read, then made undirected when the
// file is not symmetric.
alb_status alb_graph_read(const char *path, alb_host_csr *out) {
    if (!path || !out) return fail(ALB_ERR_INVALID, "alb_graph_read: bad arguments");
    std::memset(out, 0, sizeof(*out));
    const size_t len = std::strlen(path);
    auto ends = [&](const char *ext) { return len >= 4 && std::strcmp(path + len - 4, ext) == 0; };
    if (ends(".cbd")) return alb_cbd_read(path, out);
    if (!ends(".mtx"))
        return fail(ALB_ERR_UNSUPPORTED, "alb_graph_read: %s is neither .mtx nor .cbd", path);
    alb_host_csr raw;
    int32_t sym = 0;
    alb_status rc = alb_mtx_read(path, &raw, &sym);
    if (rc != ALB_OK) return rc;
    if (sym) {
        *out = raw;
        return ALB_OK;
    }
    rc = alb_csr_undirected(&raw, out);
    alb_host_csr_free(&raw);
    return rc;
}

}  // extern "C"
