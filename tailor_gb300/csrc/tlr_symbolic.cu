// tlr_symbolic.cu -- host-side nested dissection and front structures.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <string>

#include "../../include/tailor_gb300.h"
#include "tlr_symbolic.h"

namespace tlr {
namespace {

struct Box {
  int i0, i1;    // xi range [i0, i1)
  int j0, jl;    // eta interval start and length (wraps modulo nz)
  bool ring;     // the whole periodic ring
};

struct Builder {
  int ny, nz, re, leaf, slack;
  std::vector<int> lo, hi;   // symmetric xi reach per line
  std::vector<FrontInfo> &fronts;

  int add(std::vector<int> piv, std::vector<int> kids) {
    FrontInfo f;
    f.piv = std::move(piv);
    f.children = std::move(kids);
    fronts.push_back(std::move(f));
    return (int)fronts.size() - 1;
  }

  void nodes_of(const Box &b, std::vector<int> &out) {
    for (int t = 0; t < b.jl; ++t) {
      const int j = (b.j0 + t) % nz;
      for (int i = b.i0; i < b.i1; ++i) out.push_back(j * ny + i);
    }
  }

  // Returns the front index of the box's root.
  int rec(const Box &b) {
    const long long count = (long long)(b.i1 - b.i0) * b.jl;
    const int wx = b.i1 - b.i0;
    // candidate cuts and their separator sizes (nodes)
    long long best = -1;
    int kind = 0, mcut = 0, wcut = 0;
    if (count > leaf) {
      if (b.ring && b.jl > re + 1) {
        best = (long long)wx * re;
        kind = 1;
      } else if (!b.ring && b.jl >= re + 2) {
        best = (long long)wx * re;
        kind = 2;
      }
      if (wx >= 12) {
        const int m = (b.i0 + b.i1) / 2;
        int w = 0;
        for (int i = b.i0; i < m; ++i) w = std::max(w, hi[i] - m + 1);
        w = std::max(w, 1);
        if (m + w < b.i1 - 1) {
          const long long s = (long long)w * b.jl;
          if (best < 0 || s < best || (b.ring && kind == 1 && s * 100 <= best * slack)) {
            best = s;
            kind = 3;
            mcut = m;
            wcut = w;
          }
        }
      }
    }
    std::vector<int> piv;
    if (best < 0) {
      nodes_of(b, piv);
      return add(std::move(piv), {});
    }
    if (kind == 1) {  // cut the ring once: one interval child
      Box sep{b.i0, b.i1, b.j0, re, false};
      nodes_of(sep, piv);
      Box child{b.i0, b.i1, (b.j0 + re) % nz, b.jl - re, false};
      const int c = rec(child);
      return add(std::move(piv), {c});
    }
    if (kind == 2) {
      const int left = (b.jl - re) / 2;
      Box sep{b.i0, b.i1, (b.j0 + left) % nz, re, false};
      nodes_of(sep, piv);
      std::vector<int> kids;
      if (left > 0) kids.push_back(rec(Box{b.i0, b.i1, b.j0, left, false}));
      const int rl = b.jl - left - re;
      if (rl > 0) kids.push_back(rec(Box{b.i0, b.i1, (b.j0 + left + re) % nz, rl, false}));
      return add(std::move(piv), std::move(kids));
    }
    Box sep{mcut, mcut + wcut, b.j0, b.jl, false};
    nodes_of(sep, piv);
    std::vector<int> kids;
    kids.push_back(rec(Box{b.i0, mcut, b.j0, b.jl, b.ring}));
    kids.push_back(rec(Box{mcut + wcut, b.i1, b.j0, b.jl, b.ring}));
    return add(std::move(piv), std::move(kids));
  }
};

}  // namespace

int build_symbolic(int ny, int nz, const std::vector<int> &xi_idx, int sx,
                   const std::vector<int> &eta_off, int se,
                   const std::vector<int> &row_ptr, const std::vector<int> &col,
                   int leaf_nodes, Symbolic &out, int ring_slack_percent) {
  out = Symbolic{};
  out.ny = ny;
  out.nz = nz;
  out.nn = ny * nz;
  const int nn = out.nn;
  // symmetric closure of the xi coupling, as contiguous line ranges
  std::vector<int> lo(ny), hi(ny);
  for (int i = 0; i < ny; ++i) {
    lo[i] = hi[i] = i;
  }
  for (int i = 0; i < ny; ++i)
    for (int s = 0; s < sx; ++s) {
      const int ip = xi_idx[(size_t)i * sx + s];
      lo[i] = std::min(lo[i], ip); hi[i] = std::max(hi[i], ip);
      lo[ip] = std::min(lo[ip], i); hi[ip] = std::max(hi[ip], i);
    }
  int re = 0;
  for (int v : eta_off) re = std::max(re, std::abs(v));
  if (re < 1) return 1;

  Builder b{ny, nz, re, std::max(leaf_nodes, 1), ring_slack_percent, lo, hi, out.fronts};
  b.rec(Box{0, ny, 0, nz, true});
  auto &F = out.fronts;
  const int nf = (int)F.size();
  for (int t = 0; t < nf; ++t)
    for (int c : F[t].children) F[c].parent = t;
  // elimination ranks in postorder (the build order is already postorder)
  out.rank.assign(nn, -1);
  int r = 0;
  for (int t = 0; t < nf; ++t)
    for (int u : F[t].piv) out.rank[u] = r++;
  if (r != nn) return 2;
  for (int u = 0; u < nn; ++u)
    if (out.rank[u] < 0) return 3;

  // border structures, bottom-up
  std::vector<int> mark(nn, -1);
  for (int t = 0; t < nf; ++t) {
    FrontInfo &f = F[t];
    const int rmax = out.rank[f.piv.back()];
    std::vector<int> bd;
    auto consider = [&](int v) {
      if (out.rank[v] > rmax && mark[v] != t) {
        mark[v] = t;
        bd.push_back(v);
      }
    };
    for (int u : f.piv) {
      const int i = u % ny, j = u / ny;
      for (int dj = -re; dj <= re; ++dj) {
        const int jj = ((j + dj) % nz + nz) % nz;
        for (int ii = lo[i]; ii <= hi[i]; ++ii) consider(jj * ny + ii);
      }
    }
    for (int c : f.children)
      for (int v : F[c].border) consider(v);
    std::sort(bd.begin(), bd.end(),
              [&](int a, int c) { return out.rank[a] < out.rank[c]; });
    f.border = std::move(bd);
    f.p = 5 * (int)f.piv.size();
    f.m = f.p + 5 * (int)f.border.size();
    f.height = 0;
    for (int c : f.children) f.height = std::max(f.height, F[c].height + 1);
  }
  // pool layout, flops, levels
  int maxh = 0;
  for (auto &f : F) maxh = std::max(maxh, f.height);
  out.levels.assign(maxh + 1, {});
  for (int t = 0; t < nf; ++t) out.levels[F[t].height].push_back(t);
  long long off = 0, toff = 0;
  for (int h = 0; h <= maxh; ++h)
    for (int t : out.levels[h]) {
      F[t].off = off;
      F[t].toff = toff;
      off += (long long)F[t].m * F[t].m;
      toff += F[t].m;
      const double p = F[t].p, bb = F[t].m - F[t].p;
      out.flops += 8.0 * (p * p * p / 3.0 + p * p * bb + p * bb * bb);
      out.factor_elems += (long long)(p * (p + 2 * bb));
    }
  out.pool_elems = off;
  out.work_elems = toff;

  // position of each node in the front currently being built
  std::vector<int> pos(nn, -1);
  out.cmap_off.assign(nf, -1);
  out.level_entry_begin.assign(maxh + 2, 0);
  for (int h = 0; h <= maxh; ++h) {
    out.level_entry_begin[h] = (long long)out.entries.size();
    for (int t : out.levels[h]) {
      const FrontInfo &f = F[t];
      int a = 0;
      for (int u : f.piv) pos[u] = a++;
      for (int v : f.border) pos[v] = a++;
      const int rmin = out.rank[f.piv.front()], rmax = out.rank[f.piv.back()];
      // rows of the pivots: every block whose column is not eliminated yet
      for (int u : f.piv)
        for (int k = row_ptr[u]; k < row_ptr[u + 1]; ++k) {
          const int v = col[k];
          if (out.rank[v] < rmin) continue;
          if (pos[v] < 0) return 4;
          out.entries.push_back({k, pos[u], pos[v], t, v == u ? u : -1});
        }
      // columns of the pivots in border rows
      for (int v : f.border)
        for (int k = row_ptr[v]; k < row_ptr[v + 1]; ++k) {
          const int u = col[k];
          const int ru = out.rank[u];
          if (ru < rmin || ru > rmax) continue;
          out.entries.push_back({k, pos[v], pos[u], t, -1});
        }
      // maps of the children's borders into this front
      for (int c : f.children) {
        out.cmap_off[c] = (long long)out.cmap.size();
        for (int v : F[c].border) {
          if (pos[v] < 0) return 5;
          out.cmap.push_back(pos[v]);
        }
      }
      for (int u : f.piv) pos[u] = -1;
      for (int v : f.border) pos[v] = -1;
    }
  }
  out.level_entry_begin[maxh + 1] = (long long)out.entries.size();
  return 0;
}

void set_global_error(const std::string &msg);

}  // namespace tlr

extern "C" int tlr_symbolic_analyze(const tlr_rule *xi, const tlr_rule *eta, int leaf_nodes,
                                    int ring_slack_percent, tlr_symbolic_info *info,
                                    int *node_rank, int *node_front, int *front_parent,
                                    int front_capacity) {
  auto bad = [](int code, const char *msg) {
    tlr::set_global_error(msg);
    return code;
  };
  if (!xi || !eta || !info) return bad(TLR_ERR_ARG, "null argument");
  if (!xi->stencil_indices || !eta->stencil_indices || !eta->stencil_offsets)
    return bad(TLR_ERR_ARG, "FD-q rule arrays are missing");
  if (xi->periodic || !eta->periodic)
    return bad(TLR_ERR_ARG, "the xi rule must be bounded and the eta rule periodic");
  const int ny = xi->node_count, nz = eta->node_count;
  if (ny < 2 || nz < 2 || xi->q < 1 || eta->q < 1 || xi->q >= ny || eta->q >= nz)
    return bad(TLR_ERR_SIZE, "FD-q node counts or degrees out of range");
  if ((long long)ny * nz > INT_MAX / 128) return bad(TLR_ERR_SIZE, "grid too large");
  if (leaf_nodes == 0) leaf_nodes = 48;
  if (ring_slack_percent == 0) ring_slack_percent = tlr::kRingSlackDefault;
  if (leaf_nodes < 1) return bad(TLR_ERR_ARG, "leaf_nodes must be positive");
  if (ring_slack_percent < 100 || ring_slack_percent > 1000)
    return bad(TLR_ERR_ARG, "ring_slack_percent must lie in [100, 1000]");
  const int sx = xi->q + 1, se = eta->q + 1, nn = ny * nz;
  if ((long long)nn * sx * se > INT_MAX)
    return bad(TLR_ERR_SIZE, "grid and stencils too large for 32-bit pattern offsets");
  const std::vector<int> xi_idx(xi->stencil_indices, xi->stencil_indices + (size_t)ny * sx);
  const std::vector<int> eta_idx(eta->stencil_indices, eta->stencil_indices + (size_t)nz * se);
  const std::vector<int> eta_off(eta->stencil_offsets, eta->stencil_offsets + (size_t)nz * se);
  for (int v : xi_idx)
    if (v < 0 || v >= ny) return bad(TLR_ERR_STENCIL, "xi stencil index out of range");
  for (int v : eta_idx)
    if (v < 0 || v >= nz) return bad(TLR_ERR_STENCIL, "eta stencil index out of range");
  for (int v : eta_off)
    if (v <= -nz || v >= nz) return bad(TLR_ERR_STENCIL, "eta stencil offset out of range");

  // block pattern of A_bc: the tensor product of the two stencils at every
  // node, sorted and unique (the pattern tlr_assemble builds)
  std::vector<int> row_ptr((size_t)nn + 1, 0), col, cols;
  col.reserve((size_t)nn * sx * se);
  for (int u = 0; u < nn; ++u) {
    const int i = u % ny, j = u / ny;
    cols.clear();
    for (int t = 0; t < se; ++t)
      for (int s = 0; s < sx; ++s)
        cols.push_back(eta_idx[(size_t)j * se + t] * ny + xi_idx[(size_t)i * sx + s]);
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    col.insert(col.end(), cols.begin(), cols.end());
    row_ptr[u + 1] = (int)col.size();
  }
  tlr::Symbolic sym;
  const int rc = tlr::build_symbolic(ny, nz, xi_idx, sx, eta_off, se, row_ptr, col, leaf_nodes,
                                     sym, ring_slack_percent);
  if (rc) {
    char msg[64];
    std::snprintf(msg, sizeof msg, "symbolic analysis failed (code %d)", rc);
    return bad(TLR_ERR_ARG, msg);
  }
  const int nf = (int)sym.fronts.size();
  *info = tlr_symbolic_info{};
  info->fronts = nf;
  info->levels = (int)sym.levels.size();
  for (const auto &f : sym.fronts) {
    info->max_front_order = std::max(info->max_front_order, f.m);
    info->max_pivots = std::max(info->max_pivots, f.p);
  }
  info->flops = sym.flops;
  info->factor_elems = sym.factor_elems;
  info->pool_elems = sym.pool_elems;
  if (node_rank) std::copy(sym.rank.begin(), sym.rank.end(), node_rank);
  if (node_front)
    for (int t = 0; t < nf; ++t)
      for (int u : sym.fronts[t].piv) node_front[u] = t;
  if (front_parent) {
    if (front_capacity < nf)
      return bad(TLR_ERR_SIZE, "front_parent holds fewer entries than the analysis has fronts");
    for (int t = 0; t < nf; ++t) front_parent[t] = sym.fronts[t].parent;
  }
  return TLR_OK;
}
