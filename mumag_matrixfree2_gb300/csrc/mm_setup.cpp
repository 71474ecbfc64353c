// Host setup of the hot path (C++17, compiled without floating-point contraction so that sums
// follow the element order stated below on every host).
#include "mm_setup.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>

namespace mm {

static std::atomic<int> g_active_setups{0};

SetupScope::SetupScope() { g_active_setups.fetch_add(1, std::memory_order_relaxed); }
SetupScope::~SetupScope() { g_active_setups.fetch_sub(1, std::memory_order_relaxed); }

// Host threads of one parallel pass: the machine's hardware threads (at most 16) shared among the
// setups running at once, and no more than one per 4,096 items.  The thread count changes only the
// speed: every pass gives the same result for any count.
static int setup_threads(int64_t n) {
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const int active = std::max(1, g_active_setups.load(std::memory_order_relaxed));
  const int64_t budget = std::max<int64_t>(1, (int64_t)hw / active);
  const int64_t by_work = std::max<int64_t>(1, n / 4096);
  return (int)std::min<int64_t>(budget, by_work);
}

// f(t, begin, end) on contiguous chunks of [0, n), one chunk per thread (chunk t of nt in order), so
// per-chunk outputs concatenated in chunk order equal a serial loop's.  f must not throw.
template <class F>
static void parallel_chunks(int64_t n, int nt, F&& f) {
  if (nt <= 1) {
    f(0, (int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int t = 0; t < nt; ++t) th.emplace_back([&f, t, n, nt] { f(t, n * t / nt, n * (t + 1) / nt); });
  for (auto& x : th) x.join();
}

// out = the concatenation of parts (in order), each part copied by its own thread
template <class V, class P>
static void concat_parallel(const std::vector<P>& parts, V& out) {
  std::vector<size_t> off(parts.size() + 1, 0);
  for (size_t t = 0; t < parts.size(); ++t) off[t + 1] = off[t] + parts[t].size();
  out.resize(off.back());
  parallel_chunks((int64_t)parts.size(), (int)parts.size(), [&](int, int64_t t0, int64_t t1) {
    for (int64_t t = t0; t < t1; ++t) std::copy(parts[t].begin(), parts[t].end(), out.begin() + off[t]);
  });
}

// ---------------------------------------------------------------------------------------------
// geometry: orientation fix, volume, inv(J)^T and shape-function gradients (src/loop.py:56-102)
// ---------------------------------------------------------------------------------------------
static inline double det3(const double J[3][3]) {
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

void geom_compute(int N, int E, const double* knt, const int* conn_in, int* conn_out, double* volume, double* JinvT,
                  double* grad_phi) {
  for (int64_t k = 0; k < 4 * (int64_t)E; ++k)
    if (conn_in[k] < 0 || conn_in[k] >= N) throw std::runtime_error("connectivity index out of range");
  parallel_chunks(E, setup_threads(E), [&](int, int64_t e0, int64_t e1) {
  for (int e = (int)e0; e < (int)e1; ++e) {
    int c[4] = {conn_in[4 * e], conn_in[4 * e + 1], conn_in[4 * e + 2], conn_in[4 * e + 3]};
    double J[3][3];
    auto build = [&]() {
      for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 3; ++i) J[i][k] = knt[3 * c[k + 1] + i] - knt[3 * c[0] + i];
    };
    build();
    double d = det3(J);
    if (d < 0) {
      std::swap(c[1], c[2]);
      build();
      d = det3(J);
    }
    for (int a = 0; a < 4; ++a) conn_out[4 * e + a] = c[a];
    volume[e] = std::fabs(d) / 6.0;
    // inverse via the adjugate
    double inv[3][3];
    inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / d;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / d;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / d;
    inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / d;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / d;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / d;
    inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / d;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / d;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / d;
    double* T = JinvT + 9 * e;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) T[3 * i + j] = inv[j][i];
    // grad phi_a = JinvT . ghat_a with ghat_0 = (-1,-1,-1), ghat_k = e_k
    double* g = grad_phi + 12 * e;
    for (int i = 0; i < 3; ++i) {
      g[3 * 1 + i] = T[3 * i + 0];
      g[3 * 2 + i] = T[3 * i + 1];
      g[3 * 3 + i] = T[3 * i + 2];
      g[3 * 0 + i] = (-T[3 * i + 0] - T[3 * i + 1]) - T[3 * i + 2];
    }
  }
  });
}

// ---------------------------------------------------------------------------------------------
// boundary mask: nodes of faces that belong to exactly one tetrahedron (src/add_shell.py:105-136)
// ---------------------------------------------------------------------------------------------
void boundary_mask(int N, int E, const int* conn, double* mask) {
  static const int fp[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
  // faces bucketed by their smallest node: a face is on the boundary when its (b, c) pair occurs once
  // in its bucket
  // (bucket fill in parallel with relaxed atomics; every bucket is sorted before it is read, so the
  // result does not depend on the thread schedule)
  std::vector<int64_t> start((size_t)N + 1, 0);
  auto sorted_face = [&](int64_t e, int f, int& a, int& b, int& c) {
    int x = conn[4 * e + fp[f][0]], y = conn[4 * e + fp[f][1]], z = conn[4 * e + fp[f][2]];
    if (x > y) std::swap(x, y);
    if (y > z) std::swap(y, z);
    if (x > y) std::swap(x, y);
    a = x;
    b = y;
    c = z;
  };
  const int nte = setup_threads(E);
  parallel_chunks(E, nte, [&](int, int64_t e0, int64_t e1) {
    for (int64_t e = e0; e < e1; ++e)
      for (int f = 0; f < 4; ++f) {
        int a, b, c;
        sorted_face(e, f, a, b, c);
        __atomic_fetch_add(&start[(size_t)a + 1], (int64_t)1, __ATOMIC_RELAXED);
      }
  });
  for (int i = 0; i < N; ++i) start[i + 1] += start[i];
  std::vector<int64_t> fill(start.begin(), start.end() - 1);
  std::vector<std::pair<int, int>> bc((size_t)start[N]);
  parallel_chunks(E, nte, [&](int, int64_t e0, int64_t e1) {
    for (int64_t e = e0; e < e1; ++e)
      for (int f = 0; f < 4; ++f) {
        int a, b, c;
        sorted_face(e, f, a, b, c);
        bc[(size_t)__atomic_fetch_add(&fill[a], (int64_t)1, __ATOMIC_RELAXED)] = {b, c};
      }
  });
  const int nt = setup_threads(N);
  std::vector<std::vector<std::array<int, 3>>> found(nt);
  parallel_chunks(N, nt, [&](int t, int64_t n0, int64_t n1) {
    for (int64_t a = n0; a < n1; ++a) {
      auto* p0 = bc.data() + start[a];
      auto* p1 = bc.data() + start[a + 1];
      std::sort(p0, p1);
      for (auto* p = p0; p < p1;) {
        auto* q = p + 1;
        while (q < p1 && *q == *p) ++q;
        if (q - p == 1) found[t].push_back({(int)a, p->first, p->second});
        p = q;
      }
    }
  });
  for (int i = 0; i < N; ++i) mask[i] = 1.0;
  for (auto& v : found)
    for (auto& f : v) mask[f[0]] = mask[f[1]] = mask[f[2]] = 0.0;
}

// ---------------------------------------------------------------------------------------------
// Morton order of nodes and element centroids, 10 bits per axis (src/reorder_mesh.py:19-30,85-100)
// ---------------------------------------------------------------------------------------------
static inline int64_t morton30(int64_t x, int64_t y, int64_t z) {
  int64_t code = 0;
  for (int i = 0; i < 10; ++i) {
    code |= ((x >> i) & 1) << (3 * i + 2);
    code |= ((y >> i) & 1) << (3 * i + 1);
    code |= ((z >> i) & 1) << (3 * i);
  }
  return code;
}

void morton_order(int N, int E, const double* knt, const int* conn, int* node_perm, int* elem_perm) {
  double mn[3], den[3];
  for (int i = 0; i < 3; ++i) {
    double lo = knt[i], hi = knt[i];
    for (int n = 1; n < N; ++n) {
      lo = std::min(lo, knt[3 * n + i]);
      hi = std::max(hi, knt[3 * n + i]);
    }
    mn[i] = lo;
    den[i] = (hi - lo) == 0.0 ? 1.0 : (hi - lo);
  }
  auto quant = [&](double v, int i) { return (int64_t)(int32_t)(((v - mn[i]) / den[i]) * 1023.0); };
  std::vector<int64_t> key(N);
  for (int n = 0; n < N; ++n) key[n] = morton30(quant(knt[3 * n], 0), quant(knt[3 * n + 1], 1), quant(knt[3 * n + 2], 2));
  std::iota(node_perm, node_perm + N, 0);
  std::stable_sort(node_perm, node_perm + N, [&](int a, int b) { return key[a] < key[b]; });
  std::vector<int64_t> ekey(E);
  for (int e = 0; e < E; ++e) {
    double c[3];
    for (int i = 0; i < 3; ++i) {
      double s = knt[3 * conn[4 * e] + i];
      s = s + knt[3 * conn[4 * e + 1] + i];
      s = s + knt[3 * conn[4 * e + 2] + i];
      s = s + knt[3 * conn[4 * e + 3] + i];
      c[i] = s / 4.0;
    }
    ekey[e] = morton30(quant(c[0], 0), quant(c[1], 1), quant(c[2], 2));
  }
  std::iota(elem_perm, elem_perm + E, 0);
  std::stable_sort(elem_perm, elem_perm + E, [&](int a, int b) { return ekey[a] < ekey[b]; });
}

void node_graph(int N, int E, const int* conn, std::vector<int>& ptr, std::vector<int>& col) {
  // every vertex of a tetrahedron has the element's three other vertices as neighbours
  std::vector<int> cnt(N + 1, 0);
  for (int64_t k = 0; k < 4 * (int64_t)E; ++k) cnt[conn[k] + 1] += 3;
  for (int i = 0; i < N; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> raw(cnt[N]);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int e = 0; e < E; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b)
        if (a != b) raw[fill[conn[4 * e + a]]++] = conn[4 * e + b];
  ptr.assign(N + 1, 0);
  parallel_chunks(N, setup_threads(N), [&](int, int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
      std::sort(raw.begin() + cnt[i], raw.begin() + cnt[i + 1]);
      const auto end = std::unique(raw.begin() + cnt[i], raw.begin() + cnt[i + 1]);
      ptr[i + 1] = (int)(end - (raw.begin() + cnt[i]));
    }
  });
  for (int i = 0; i < N; ++i) ptr[i + 1] += ptr[i];
  col.resize(ptr[N]);
  parallel_chunks(N, setup_threads(N), [&](int, int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i)
      std::copy(raw.begin() + cnt[i], raw.begin() + cnt[i] + (ptr[i + 1] - ptr[i]), col.begin() + ptr[i]);
  });
}

void rcm_order(int N, const std::vector<int>& ptr, const std::vector<int>& col, const int* seeds, int* perm) {
  std::vector<int> order(N);
  std::vector<char> seen(N, 0);
  auto deg = [&](int v) { return ptr[v + 1] - ptr[v]; };
  int n = 0;
  for (int z = 0; z < N && n < N; ++z) {
    const int seed = seeds[z];
    if (seen[seed]) continue;
    seen[seed] = 1;
    order[n++] = seed;
    for (int head = n - 1; head < n; ++head) {  // the queue is order[head .. n)
      const int v = order[head];
      const int first = n;
      for (int k = ptr[v]; k < ptr[v + 1]; ++k) {
        const int u = col[k];
        if (!seen[u]) {
          seen[u] = 1;
          order[n++] = u;
        }
      }
      std::stable_sort(order.begin() + first, order.begin() + n, [&](int a, int b) { return deg(a) < deg(b); });
    }
  }
  for (int i = 0; i < N; ++i) perm[i] = order[N - 1 - i];
}

// ---------------------------------------------------------------------------------------------
// assembly helpers
// ---------------------------------------------------------------------------------------------
struct NodeElems {
  std::vector<int> ptr, elem;
};

// Node -> element lists, each in ascending element order (the order an element loop visits them):
// counts and slots taken with relaxed atomics over element chunks in parallel, then every node's list
// sorted, so the result does not depend on the thread schedule.
static NodeElems node_elements(int N, int E, const int* conn, const std::vector<char>* use = nullptr) {
  NodeElems ne;
  ne.ptr.assign(N + 1, 0);
  const int nte = setup_threads(E);
  int* cnt = ne.ptr.data() + 1;
  parallel_chunks(E, nte, [&](int, int64_t e0, int64_t e1) {
    for (int64_t e = e0; e < e1; ++e) {
      if (use && !(*use)[e]) continue;
      for (int a = 0; a < 4; ++a) __atomic_fetch_add(&cnt[conn[4 * e + a]], 1, __ATOMIC_RELAXED);
    }
  });
  for (int i = 0; i < N; ++i) ne.ptr[i + 1] += ne.ptr[i];
  ne.elem.resize(ne.ptr[N]);
  std::vector<int> fill(ne.ptr.begin(), ne.ptr.end() - 1);
  parallel_chunks(E, nte, [&](int, int64_t e0, int64_t e1) {
    for (int64_t e = e0; e < e1; ++e) {
      if (use && !(*use)[e]) continue;
      for (int a = 0; a < 4; ++a) ne.elem[__atomic_fetch_add(&fill[conn[4 * e + a]], 1, __ATOMIC_RELAXED)] = (int)e;
    }
  });
  parallel_chunks(N, setup_threads(N), [&](int, int64_t n0, int64_t n1) {
    for (int64_t i = n0; i < n1; ++i) std::sort(ne.elem.begin() + ne.ptr[i], ne.elem.begin() + ne.ptr[i + 1]);
  });
  return ne;
}

static inline double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static inline int find_col(const int* cols, int n, int c) {
  const int* p = std::lower_bound(cols, cols + n, c);
  return (int)(p - cols);
}

// Drop exactly-zero entries (scipy's CSR arithmetic keeps only non-zero results).
static void drop_zeros(HostCSR& A) {
  int w = 0;
  std::vector<int> nptr(A.n_rows + 1, 0);
  for (int r = 0; r < A.n_rows; ++r) {
    for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k)
      if (A.val[k] != 0.0) {
        A.col[w] = A.col[k];
        A.val[w] = A.val[k];
        ++w;
      }
    nptr[r + 1] = w;
  }
  A.ptr = nptr;
  A.col.resize(w);
  A.val.resize(w);
}

// local index of node i in element e
static inline int local_index(const int* conn, int e, int i) {
  return conn[4 * e] == i ? 0 : conn[4 * e + 1] == i ? 1 : conn[4 * e + 2] == i ? 2 : 3;
}

HostCSR assemble_poisson(int N, int E, const int* conn, const double* volume, const double* gp, const double* mask,
                         double reg) {
  NodeElems ne = node_elements(N, E, conn);
  HostCSR A;
  A.n_rows = A.n_cols = N;
  A.ptr.assign(N + 1, 0);
  const int nt = setup_threads(N);
  std::vector<std::vector<int>> tcol(nt);
  parallel_chunks(N, nt, [&](int t, int64_t r0, int64_t r1) {
    std::vector<int> tmp;
    for (int i = (int)r0; i < (int)r1; ++i) {
      tmp.clear();
      for (int k = ne.ptr[i]; k < ne.ptr[i + 1]; ++k) {
        int e = ne.elem[k];
        for (int b = 0; b < 4; ++b) tmp.push_back(conn[4 * e + b]);
      }
      tmp.push_back(i);
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      A.ptr[i + 1] = (int)tmp.size();
      tcol[t].insert(tcol[t].end(), tmp.begin(), tmp.end());
    }
  });
  for (int i = 0; i < N; ++i) A.ptr[i + 1] += A.ptr[i];
  concat_parallel(tcol, A.col);
  A.val.resize(A.col.size());
  // K_ab = sum_e Ve (grad phi_a . grad phi_b): row by row over the row's elements in ascending order,
  // which is the order an element loop adds them in
  parallel_chunks(N, nt, [&](int, int64_t r0, int64_t r1) {
    for (int r = (int)r0; r < (int)r1; ++r) {
      const int* rc = A.col.data() + A.ptr[r];
      const int rn = A.ptr[r + 1] - A.ptr[r];
      std::fill(A.val.begin() + A.ptr[r], A.val.begin() + A.ptr[r + 1], 0.0);
      for (int k = ne.ptr[r]; k < ne.ptr[r + 1]; ++k) {
        const int e = ne.elem[k];
        const double* g = gp + 12 * e;
        const int a = local_index(conn, e, r);
        for (int b = 0; b < 4; ++b) {
          int pos = find_col(rc, rn, conn[4 * e + b]);
          A.val[A.ptr[r] + pos] += volume[e] * dot3(g + 3 * a, g + 3 * b);
        }
      }
    }
  });
  if (mask) {
    for (int r = 0; r < N; ++r)
      for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k)
        if (mask[r] == 0.0 || mask[A.col[k]] == 0.0) A.val[k] = 0.0;
  }
  for (int r = 0; r < N; ++r) {
    int pos = find_col(A.col.data() + A.ptr[r], A.ptr[r + 1] - A.ptr[r], r);
    A.val[A.ptr[r] + pos] += reg;
    if (mask && mask[r] == 0.0) A.val[A.ptr[r] + pos] = 1.0;
  }
  drop_zeros(A);
  return A;
}

EnergyOp assemble_energy(int N, int E, const int* conn, const double* volume, const double* gp, const int* mat_id,
                         int n_mat, const double* Alu, const double* K1lu, const double* Jslu, const double* k_easy) {
  EnergyOp op;
  op.n_mat = n_mat;
  std::vector<char> use(E, 0);
  std::vector<char> mat_used(n_mat, 0);
  for (int e = 0; e < E; ++e) {
    int g = mat_id[e] - 1;
    if (g < 0 || g >= n_mat) throw std::runtime_error("material id out of range");
    if (Alu[g] != 0.0 || K1lu[g] != 0.0 || Jslu[g] != 0.0) {
      use[e] = 1;
      mat_used[g] = 1;
    }
  }
  // single easy axis when every material that carries anisotropy shares one axis
  int first = -1;
  op.single_axis = true;
  for (int g = 0; g < n_mat; ++g) {
    if (!mat_used[g] || K1lu[g] == 0.0) continue;
    if (first < 0) first = g;
    else if (k_easy[3 * g] != k_easy[3 * first] || k_easy[3 * g + 1] != k_easy[3 * first + 1] ||
             k_easy[3 * g + 2] != k_easy[3 * first + 2])
      op.single_axis = false;
  }
  NodeElems ne = node_elements(N, E, conn, &use);
  op.diag_exchange.assign(N, 0.0);
  // pattern: per node with used elements, the sorted unique (column, axis group) keys; chunks in parallel
  const int nt = setup_threads(N);
  std::vector<int> len(N, -1);
  std::vector<std::vector<std::pair<int, int>>> tkeys(nt);
  parallel_chunks(N, nt, [&](int t, int64_t n0, int64_t n1) {
    std::vector<std::pair<int, int>> keys;
    for (int i = (int)n0; i < (int)n1; ++i) {
      if (ne.ptr[i + 1] == ne.ptr[i]) continue;
      keys.clear();
      for (int k = ne.ptr[i]; k < ne.ptr[i + 1]; ++k) {
        int e = ne.elem[k];
        int g = op.single_axis ? 0 : mat_id[e] - 1;
        for (int b = 0; b < 4; ++b) keys.emplace_back(conn[4 * e + b], g);
      }
      std::sort(keys.begin(), keys.end());
      keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
      len[i] = (int)keys.size();
      tkeys[t].insert(tkeys[t].end(), keys.begin(), keys.end());
    }
  });
  op.ptr.push_back(0);
  for (int i = 0; i < N; ++i)
    if (len[i] >= 0) {
      op.rows.push_back(i);
      op.ptr.push_back(op.ptr.back() + len[i]);
    }
  {
    std::vector<size_t> off(nt + 1, 0);
    for (int t = 0; t < nt; ++t) off[t + 1] = off[t] + tkeys[t].size();
    op.col.resize(off[nt]);
    op.mat.resize(off[nt]);
    parallel_chunks(nt, nt, [&](int, int64_t t0, int64_t t1) {
      for (int64_t t = t0; t < t1; ++t)
        for (size_t k = 0; k < tkeys[t].size(); ++k) {
          op.col[off[t] + k] = tkeys[t][k].first;
          op.mat[off[t] + k] = tkeys[t][k].second;
        }
    });
  }
  op.n_rows = (int)op.rows.size();
  size_t nnz = op.col.size();
  for (dvec* v : {&op.w, &op.q, &op.gx, &op.gy, &op.gz, &op.dx, &op.dy, &op.dz}) v->resize(nnz);
  // values row by row over the row's used elements in ascending order (the order an element loop adds
  // them in), one row per node, rows in parallel
  parallel_chunks(op.n_rows, setup_threads(op.n_rows), [&](int, int64_t r0, int64_t r1) {
    for (int r = (int)r0; r < (int)r1; ++r) {
      const int node = op.rows[r];
      const int base = op.ptr[r], n = op.ptr[r + 1] - base;
      for (dvec* v : {&op.w, &op.q, &op.gx, &op.gy, &op.gz, &op.dx, &op.dy, &op.dz})
        std::fill(v->begin() + base, v->begin() + base + n, 0.0);
      for (int kk = ne.ptr[node]; kk < ne.ptr[node + 1]; ++kk) {
        const int e = ne.elem[kk];
        const int g = mat_id[e] - 1;
        const int gk = op.single_axis ? 0 : g;
        const double* G = gp + 12 * e;
        const double cA = 2.0 * Alu[g] * volume[e];
        const double cK = 2.0 * K1lu[g] * volume[e] / 20.0;
        const double cG = 2.0 * Jslu[g] * volume[e] / 4.0;
        const double cD = Jslu[g] * volume[e] / 4.0;
        const int a = local_index(conn, e, node);
        op.diag_exchange[node] += cA * dot3(G + 3 * a, G + 3 * a);
        for (int b = 0; b < 4; ++b) {
          const int cb = conn[4 * e + b];
          // entries are sorted by (col, group): find the matching pair
          int lo = 0, hi = n;
          while (lo < hi) {
            int mid = (lo + hi) / 2;
            int mc = op.col[base + mid], mg = op.mat[base + mid];
            if (mc < cb || (mc == cb && mg < gk)) lo = mid + 1;
            else hi = mid;
          }
          const int k = base + lo;
          op.w[k] += cA * dot3(G + 3 * a, G + 3 * b);
          op.q[k] += cK * (a == b ? 2.0 : 1.0);
          op.gx[k] += cG * G[3 * b + 0];
          op.gy[k] += cG * G[3 * b + 1];
          op.gz[k] += cG * G[3 * b + 2];
          op.dx[k] += cD * G[3 * a + 0];
          op.dy[k] += cD * G[3 * a + 1];
          op.dz[k] += cD * G[3 * a + 2];
        }
      }
    }
  });
  if (op.single_axis) {
    // all entries refer to the shared axis; remember which material carries it
    for (auto& m : op.mat) m = first < 0 ? 0 : first;
  }
  return op;
}

// ---------------------------------------------------------------------------------------------
// smoothed aggregation (the project's own algorithm; restated by the oracle for parity)
// ---------------------------------------------------------------------------------------------
static HostCSR transpose(const HostCSR& A) {
  HostCSR T;
  T.n_rows = A.n_cols;
  T.n_cols = A.n_rows;
  T.ptr.assign(T.n_rows + 1, 0);
  for (int c : A.col) T.ptr[c + 1]++;
  for (int i = 0; i < T.n_rows; ++i) T.ptr[i + 1] += T.ptr[i];
  T.col.resize(A.col.size());
  T.val.resize(A.col.size());
  std::vector<int> fill(T.ptr.begin(), T.ptr.end() - 1);
  for (int r = 0; r < A.n_rows; ++r)
    for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k) {
      int p = fill[A.col[k]]++;
      T.col[p] = r;
      T.val[p] = A.val[k];
    }
  return T;
}

// C = A * B (Gustavson), sums in the order of A's sorted columns; exact zeros dropped; columns sorted.
static HostCSR spgemm(const HostCSR& A, const HostCSR& B) {
  HostCSR C;
  C.n_rows = A.n_rows;
  C.n_cols = B.n_cols;
  C.ptr.assign(C.n_rows + 1, 0);
  const int nt = setup_threads(A.n_rows);
  std::vector<std::vector<int>> tcol(nt), tlen(nt);
  std::vector<std::vector<double>> tval(nt);
  // rows in chunks; each row's products are summed in the order of a serial loop
  parallel_chunks(A.n_rows, nt, [&](int t, int64_t r0, int64_t r1) {
    std::vector<double> acc(B.n_cols, 0.0);
    std::vector<int> mark(B.n_cols, -1), cols;
    for (int i = (int)r0; i < (int)r1; ++i) {
      cols.clear();
      for (int ka = A.ptr[i]; ka < A.ptr[i + 1]; ++ka) {
        int k = A.col[ka];
        double a = A.val[ka];
        for (int kb = B.ptr[k]; kb < B.ptr[k + 1]; ++kb) {
          int j = B.col[kb];
          if (mark[j] != i) {
            mark[j] = i;
            acc[j] = 0.0;
            cols.push_back(j);
          }
          acc[j] += a * B.val[kb];
        }
      }
      std::sort(cols.begin(), cols.end());
      int len = 0;
      for (int j : cols)
        if (acc[j] != 0.0) {
          tcol[t].push_back(j);
          tval[t].push_back(acc[j]);
          ++len;
        }
      tlen[t].push_back(len);
    }
  });
  int r = 0;
  for (int t = 0; t < nt; ++t)
    for (int len : tlen[t]) {
      C.ptr[r + 1] = C.ptr[r] + len;
      ++r;
    }
  concat_parallel(tcol, C.col);
  concat_parallel(tval, C.val);
  return C;
}

HostCSR fused_restriction(const HostCSR& R, const HostCSR& A, const std::vector<double>& s) {
  HostCSR AS;
  AS.n_rows = A.n_rows;
  AS.n_cols = A.n_cols;
  AS.ptr = A.ptr;
  AS.col.resize(A.col.size());
  AS.val.resize(A.val.size());
  parallel_chunks((int64_t)A.col.size(), setup_threads(A.n_rows), [&](int, int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; ++k) {
      AS.col[k] = A.col[k];
      AS.val[k] = A.val[k] * s[A.col[k]];
    }
  });
  const HostCSR C = spgemm(R, AS);
  HostCSR F;
  F.n_rows = R.n_rows;
  F.n_cols = R.n_cols;
  F.ptr.assign(F.n_rows + 1, 0);
  F.col.reserve(C.col.size() + R.col.size());
  F.val.reserve(C.col.size() + R.col.size());
  for (int i = 0; i < R.n_rows; ++i) {  // F = R - C, merging two sorted rows
    int a = R.ptr[i], b = C.ptr[i];
    const int ae = R.ptr[i + 1], be = C.ptr[i + 1];
    while (a < ae || b < be) {
      const int ca = a < ae ? R.col[a] : R.n_cols;
      const int cb = b < be ? C.col[b] : R.n_cols;
      const int c = std::min(ca, cb);
      double v = 0.0;
      if (ca == c) v += R.val[a++];
      if (cb == c) v -= C.val[b++];
      if (v != 0.0) {
        F.col.push_back(c);
        F.val.push_back(v);
      }
    }
    F.ptr[i + 1] = (int)F.col.size();
  }
  return F;
}

HostCSR fused_restriction_ra(const HostCSR& R, const HostCSR& RA, const std::vector<double>& s) {
  const int n = R.n_rows;
  std::vector<int> cnt(n + 1, 0);
  std::vector<std::vector<int>> tcol;
  std::vector<std::vector<double>> tval;
  const int nt = setup_threads(RA.ptr[n]);
  tcol.resize(nt);
  tval.resize(nt);
  // F = R - RA diag(s), merging two sorted rows, exact zeros dropped; rows in chunks, concatenated in order
  parallel_chunks(n, nt, [&](int t, int64_t r0, int64_t r1) {
    for (int64_t i = r0; i < r1; ++i) {
      int a = R.ptr[i], b = RA.ptr[i], len = 0;
      const int ae = R.ptr[i + 1], be = RA.ptr[i + 1];
      while (a < ae || b < be) {
        const int ca = a < ae ? R.col[a] : R.n_cols;
        const int cb = b < be ? RA.col[b] : R.n_cols;
        const int c = std::min(ca, cb);
        double v = 0.0;
        if (ca == c) v += R.val[a++];
        if (cb == c) v -= RA.val[b++] * s[c];
        if (v != 0.0) {
          tcol[t].push_back(c);
          tval[t].push_back(v);
          ++len;
        }
      }
      cnt[i + 1] = len;
    }
  });
  HostCSR F;
  F.n_rows = n;
  F.n_cols = R.n_cols;
  F.ptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) F.ptr[i + 1] = F.ptr[i] + cnt[i + 1];
  concat_parallel(tcol, F.col);
  concat_parallel(tval, F.val);
  return F;
}

static std::vector<double> diag_of(const HostCSR& A) {
  std::vector<double> d(A.n_rows, 0.0);
  parallel_chunks(A.n_rows, setup_threads(A.n_rows), [&](int, int64_t r0, int64_t r1) {
    for (int64_t r = r0; r < r1; ++r)
      for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k)
        if (A.col[k] == r) d[r] = A.val[k];
  });
  return d;
}

static std::vector<double> spai0_of(const HostCSR& A, const std::vector<double>& d) {
  std::vector<double> s(A.n_rows);
  parallel_chunks(A.n_rows, setup_threads(A.n_rows), [&](int, int64_t r0, int64_t r1) {
    for (int64_t r = r0; r < r1; ++r) {
      double ss = 0.0;
      for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k) ss += A.val[k] * A.val[k];
      s[r] = d[r] / (ss + 1e-30);
    }
  });
  return s;
}

static std::vector<int> aggregate(const HostCSR& A, const std::vector<double>& d, double theta, int& nagg) {
  int n = A.n_rows;
  const double t2 = theta * theta;
  // strength pattern
  std::vector<int> sptr(n + 1, 0), scol;
  for (int i = 0; i < n; ++i) {
    for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
      int j = A.col[k];
      double v = A.val[k];
      if (j != i && v * v > t2 * std::fabs(d[i] * d[j])) scol.push_back(j);
    }
    sptr[i + 1] = (int)scol.size();
  }
  std::vector<int> agg(n, -1);
  nagg = 0;
  for (int i = 0; i < n; ++i) {  // pass 1
    if (agg[i] >= 0 || sptr[i + 1] == sptr[i]) continue;
    bool free_nb = true;
    for (int k = sptr[i]; k < sptr[i + 1]; ++k)
      if (agg[scol[k]] >= 0) {
        free_nb = false;
        break;
      }
    if (!free_nb) continue;
    agg[i] = nagg;
    for (int k = sptr[i]; k < sptr[i + 1]; ++k) agg[scol[k]] = nagg;
    ++nagg;
  }
  std::vector<int> after1 = agg;
  for (int i = 0; i < n; ++i) {  // pass 2
    if (after1[i] >= 0) continue;
    for (int k = sptr[i]; k < sptr[i + 1]; ++k)
      if (after1[scol[k]] >= 0) {
        agg[i] = after1[scol[k]];
        break;
      }
  }
  for (int i = 0; i < n; ++i) {  // pass 3
    if (agg[i] >= 0 || sptr[i + 1] == sptr[i]) continue;
    agg[i] = nagg;
    for (int k = sptr[i]; k < sptr[i + 1]; ++k)
      if (agg[scol[k]] < 0) agg[scol[k]] = nagg;
    ++nagg;
  }
  return agg;
}

void assemble_magnetoelastic(EnergyOp& op, int N, int E, const int* conn, const double* volume, const int* mat_id,
                             int n, const double* k1me, const double* k1me_p) {
  if (n < 0 || n > E) throw std::runtime_error("magnetoelastic arrays longer than the element count");
  op.mx.assign(op.col.size(), 0.0);
  op.my.assign(op.col.size(), 0.0);
  std::vector<int> row_of(N, -1);
  for (int r = 0; r < op.n_rows; ++r) row_of[op.rows[r]] = r;
  for (int e = 0; e < n; ++e) {
    const double kp = k1me_p ? k1me_p[e] : 0.0;
    const double cx = 2.0 * (k1me[e] + kp) * volume[e] / 20.0;
    const double cy = 2.0 * (k1me[e] - kp) * volume[e] / 20.0;
    if (cx == 0.0 && cy == 0.0) continue;
    const int gk = mat_id[e] - 1;  // entry group of a multi-axis operator
    for (int a = 0; a < 4; ++a) {
      const int r = row_of[conn[4 * e + a]];
      if (r < 0) throw std::runtime_error("magnetoelastic constant on an element outside the magnetic region");
      const int base = op.ptr[r], len = op.ptr[r + 1] - base;
      for (int b = 0; b < 4; ++b) {
        const int cb = conn[4 * e + b];
        int k = -1;
        for (int t = 0; t < len; ++t)
          if (op.col[base + t] == cb && (op.single_axis || op.mat[base + t] == gk)) {
            k = base + t;
            break;
          }
        if (k < 0) throw std::runtime_error("magnetoelastic entry outside the operator's pattern");
        op.mx[k] += cx * (a == b ? 2.0 : 1.0);
        op.my[k] += cy * (a == b ? 2.0 : 1.0);
      }
    }
  }
}

// rho(D^-1 A) by the power method from a fixed pseudo-random start (Knuth's multiplicative hash of the
// row index), `steps` products, times `safety` (the method approaches rho from below).  Row sums in
// column order (threaded by rows) and norms as left-to-right serial sums, so that a numpy
// restatement with cumulative sums reproduces the estimate.
static double power_rho(const HostCSR& A, const std::vector<double>& d, int steps, double safety) {
  const int n = A.n_rows;
  if (n == 0) return 1.0;
  std::vector<double> dinv(n), x(n), y(n);
  for (int i = 0; i < n; ++i) {
    dinv[i] = d[i] != 0.0 ? 1.0 / d[i] : 0.0;
    x[i] = (double)(((uint64_t)i * 2654435761ull) % 4294967296ull) / 4294967296.0 - 0.5;
  }
  auto norm = [](const std::vector<double>& v) {
    double s = 0.0;
    for (double e : v) s += e * e;
    return std::sqrt(s);
  };
  double nx = norm(x), lam = 1.0;
  const int nt = setup_threads(A.ptr[n]);
  for (int s = 0; s < steps; ++s) {
    parallel_chunks(n, nt, [&](int, int64_t r0, int64_t r1) {
      for (int64_t i = r0; i < r1; ++i) {
        double acc = 0.0;
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) acc += A.val[k] * x[A.col[k]];
        y[i] = dinv[i] * acc;
      }
    });
    const double ny = norm(y);
    if (!(ny > 0.0 && nx > 0.0)) break;
    lam = ny / nx;
    for (int i = 0; i < n; ++i) x[i] = y[i] / ny;
    nx = 1.0;
  }
  return safety * lam;
}

// The level-1 operator without its weak couplings: an off-diagonal a_ij is weak when
// |a_ij| + |a_ji| < 2 eps sqrt(|a_ii a_jj|) (symmetric in i and j; a_ji is 0 when not stored), and each
// row's weak values, summed from zero in column order, are added to its diagonal, so that the row
// sums (the operator's action on constants, which smoothed aggregation interpolates) stay as they
// were.  The Galerkin operator of the smoothed prolongator carries a long tail of such couplings
// (76 entries per row on the 80 nm cube, most of them below 0.002 of the diagonal scale).
static HostCSR filter_weak(const HostCSR& A, double eps) {
  const int n = A.n_rows;
  const std::vector<double> d = diag_of(A);
  auto value_at = [&](int r, int c) {
    const int* b = A.col.data() + A.ptr[r];
    const int* e = A.col.data() + A.ptr[r + 1];
    const int* p = std::lower_bound(b, e, c);
    return (p != e && *p == c) ? A.val[p - A.col.data()] : 0.0;
  };
  std::vector<char> weak(A.col.size(), 0);
  std::vector<double> lump(n, 0.0);
  std::vector<int> cnt(n + 1, 0);
  parallel_chunks(n, setup_threads(A.ptr[n]), [&](int, int64_t r0, int64_t r1) {
    for (int64_t i = r0; i < r1; ++i) {
      double l = 0.0;
      int kept = 0;
      for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
        const int j = A.col[k];
        const bool w = j != i && std::fabs(A.val[k]) + std::fabs(value_at(j, (int)i)) <
                                     2.0 * eps * std::sqrt(std::fabs(d[i] * d[j]));
        weak[k] = w ? 1 : 0;
        if (w) l += A.val[k];
        else ++kept;
      }
      lump[i] = l;
      cnt[i + 1] = kept;
    }
  });
  HostCSR B;
  B.n_rows = n;
  B.n_cols = A.n_cols;
  B.ptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) B.ptr[i + 1] = B.ptr[i] + cnt[i + 1];
  B.col.resize(B.ptr[n]);
  B.val.resize(B.ptr[n]);
  parallel_chunks(n, setup_threads(A.ptr[n]), [&](int, int64_t r0, int64_t r1) {
    for (int64_t i = r0; i < r1; ++i) {
      int w = B.ptr[i];
      for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
        if (weak[k]) continue;
        B.col[w] = A.col[k];
        B.val[w] = A.col[k] == i ? A.val[k] + lump[i] : A.val[k];
        ++w;
      }
    }
  });
  return B;
}

static std::vector<AmgLevel> build_amg_theta(const HostCSR& A0, const AmgParams& prm, double theta0) {
  std::vector<AmgLevel> levels;
  levels.reserve(prm.max_levels);
  HostCSR next = A0;
  double theta = theta0;
  while (true) {
    levels.emplace_back();
    AmgLevel& L = levels.back();
    L.A = std::move(next);
    const HostCSR& Acur = L.A;
    L.diag = diag_of(Acur);
    L.spai0 = spai0_of(Acur, L.diag);
    int n = Acur.n_rows;
    if (n <= prm.max_coarse || (int)levels.size() >= prm.max_levels) break;
    int nagg = 0;
    std::vector<int> agg = aggregate(Acur, levels.back().diag, theta, nagg);
    if (nagg == 0 || nagg >= n) break;
    // tentative prolongator
    std::vector<int> size(nagg, 0);
    for (int a : agg)
      if (a >= 0) size[a]++;
    HostCSR T;
    T.n_rows = n;
    T.n_cols = nagg;
    T.ptr.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
      if (agg[i] >= 0) {
        T.col.push_back(agg[i]);
        T.val.push_back(1.0 / std::sqrt((double)size[agg[i]]));
      }
      T.ptr[i + 1] = (int)T.col.size();
    }
    // damped-Jacobi smoothing with omega = (4/3) / rho(D^-1 A)
    const std::vector<double>& d = levels.back().diag;
    const double rho = power_rho(Acur, d, prm.rho_steps, prm.rho_safety);
    double omega = (4.0 / 3.0) / rho;
    HostCSR AT = spgemm(Acur, T);
    HostCSR P;
    P.n_rows = n;
    P.n_cols = nagg;
    P.ptr.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
      double dinv = d[i] != 0.0 ? 1.0 / d[i] : 0.0;
      int ka = AT.ptr[i], kt = T.ptr[i];
      while (ka < AT.ptr[i + 1] || kt < T.ptr[i + 1]) {
        int ca = ka < AT.ptr[i + 1] ? AT.col[ka] : INT32_MAX;
        int ct = kt < T.ptr[i + 1] ? T.col[kt] : INT32_MAX;
        int c = std::min(ca, ct);
        double tv = (ct == c) ? T.val[kt++] : 0.0;
        double av = (ca == c) ? AT.val[ka++] : 0.0;
        double v = tv - omega * (dinv * av);
        if (v != 0.0) {
          P.col.push_back(c);
          P.val.push_back(v);
        }
      }
      P.ptr[i + 1] = (int)P.col.size();
    }
    HostCSR R = transpose(P);
    HostCSR RA = spgemm(R, Acur);
    next = spgemm(RA, P);
    L.RA = std::move(RA);
    if (levels.size() == 1 && prm.filter_eps > 0.0) next = filter_weak(next, prm.filter_eps);
    L.P = std::move(P);
    L.R = std::move(R);
    L.agg = std::move(agg);
    theta *= prm.theta_factor;
  }
  return levels;
}

std::vector<AmgLevel> build_amg(const HostCSR& A0, const AmgParams& prm) {
  if (prm.theta0 > 0.0) return build_amg_theta(A0, prm, prm.theta0);
  std::vector<AmgLevel> levels = build_amg_theta(A0, prm, 0.115);
  if (levels.size() > 4) levels = build_amg_theta(A0, prm, 0.1);
  return levels;
}

std::vector<double> dense_inverse(const HostCSR& A) {
  int n = A.n_rows;
  std::vector<double> M((size_t)n * n, 0.0), I((size_t)n * n, 0.0);
  for (int r = 0; r < n; ++r) {
    for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k) M[(size_t)r * n + A.col[k]] = A.val[k];
    I[(size_t)r * n + r] = 1.0;
  }
  for (int c = 0; c < n; ++c) {  // Gauss-Jordan with partial pivoting
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(M[(size_t)r * n + c]) > std::fabs(M[(size_t)piv * n + c])) piv = r;
    if (M[(size_t)piv * n + c] == 0.0) throw std::runtime_error("coarsest AMG matrix is singular");
    if (piv != c)
      for (int k = 0; k < n; ++k) {
        std::swap(M[(size_t)c * n + k], M[(size_t)piv * n + k]);
        std::swap(I[(size_t)c * n + k], I[(size_t)piv * n + k]);
      }
    double inv = 1.0 / M[(size_t)c * n + c];
    for (int k = 0; k < n; ++k) {
      M[(size_t)c * n + k] *= inv;
      I[(size_t)c * n + k] *= inv;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = M[(size_t)r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        M[(size_t)r * n + k] -= f * M[(size_t)c * n + k];
        I[(size_t)r * n + k] -= f * I[(size_t)c * n + k];
      }
    }
  }
  return I;
}

}  // namespace mm
