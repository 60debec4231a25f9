// Synthetic graph generators and CSR assembly (host, OpenMP).
//
// The reference reads its inputs from files (bfs/src/biio.h:21-149) and, for
// undirected use, merges a CSR with its transpose (bfs/src/main.c:130-169,
// bfs/src/utils.c:351-379). Here the same end state -- a symmetric CSR with
// ascending, duplicate-free rows -- is produced from generated edge lists.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <new>
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
