// C ABI (include/sayaka_gb300.h) over the host tree mirror and the GPU MAC
// solver.  Converts between the reference's TreeData buffer layout and the
// compact device layout, validates inputs and turns failures into status codes.
#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <functional>
#include <mutex>
#include <memory>
#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sayaka_gb300.h"
#include "mac_solver.h"
#include "tower.h"
#include "tree.h"

using namespace sayaka_gb300;

struct sayaka_tree {
  AmrTree t;
  // SoA export of the current tree (refreshed on demand)
  std::vector<int32_t> level, neighbor, child, parent, wc, nt;
  std::vector<double> len;
  std::vector<Tower> towers;
  bool dirty = true;
};

struct sayaka_mac {
  std::unique_ptr<MacGpu> gpu;
  std::string err;
  double *pinned = nullptr;  // staging for TreeData-layout transfers
  size_t pinned_n = 0;
  ~sayaka_mac() {
    if (pinned) cudaFreeHost(pinned);
  }
};

namespace {

void refresh(sayaka_tree *h) {
  if (!h->dirty) return;
  const AmrTree &t = h->t;
  const int n = t.num_blocks;
  h->level.resize(n);
  h->neighbor.resize((size_t)n * 6);
  h->child.resize((size_t)n * 8);
  h->parent.resize(n);
  h->wc.resize(n);
  h->nt.resize(n);
  h->len.resize((size_t)n * 3);
  for (int b = 0; b < n; b++) {
    const TreeNode &x = t.nodes[b];
    h->level[b] = x.level;
    for (int f = 0; f < 6; f++) h->neighbor[b * 6 + f] = x.neighbor[f];
    for (int c = 0; c < 8; c++) h->child[b * 8 + c] = x.child[c];
    h->parent[b] = x.parent;
    h->wc[b] = x.which_child;
    h->nt[b] = x.node_type;
    for (int d = 0; d < 3; d++) h->len[b * 3 + d] = x.length[d];
  }
  h->towers = build_towers(t);
  h->dirty = false;
}

// TreeData layout of cell data (stag < 0) or face data of direction stag
struct Layout {
  int nd, nb, ncomp, g, comp, stag;
  long G[3];
  long cap;
  Layout(int nd_, int nb_, int ncomp_, int g_, int comp_, int stag_)
      : nd(nd_), nb(nb_), ncomp(ncomp_), g(g_), comp(comp_), stag(stag_) {
    for (int d = 0; d < 3; d++) G[d] = d < nd ? nb + (d == stag) + 2 * g : 1;
    cap = G[0] * G[1] * G[2];
  }
  long at(int b, int i, int j, int k) const {
    const long gz = nd == 3 ? g : 0;
    return (long)b * cap * ncomp + (long)comp * cap + (i + g) + G[0] * ((j + g) + G[1] * (k + gz));
  }
  bool ok() const { return ncomp >= 1 && comp >= 0 && comp < ncomp && g >= 0; }
};

// Persistent host workers for the TreeData <-> compact copies: created on
// first use and reused by every call (spawning threads per call costs as
// much as copying a few MB); one job at a time, the caller takes part.
class HostPool {
 public:
  static HostPool &get() {
    static HostPool *pool = new HostPool();  // never destroyed: workers end with the process
    return *pool;
  }
  int size() const { return (int)workers_.size() + 1; }
  // task(i) for i in [0, n), on the workers and the calling thread
  void run(int n, const std::function<void(int)> &task) {
    std::lock_guard<std::mutex> one_job(job_mu_);
    {
      std::lock_guard<std::mutex> lk(mu_);
      task_ = &task;
      n_ = n;
      next_.store(0);
      busy_ = (int)workers_.size();
      gen_++;
    }
    cv_.notify_all();
    drain();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return busy_ == 0; });
    task_ = nullptr;
  }

 private:
  HostPool() {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nw = (int)std::min<unsigned>(16u, hw) - 1;
    for (int i = 0; i < nw; i++) workers_.emplace_back([this] { loop(); });
    for (auto &w : workers_) w.detach();
  }
  void drain() {
    for (int i = next_.fetch_add(1); i < n_; i = next_.fetch_add(1)) (*task_)(i);
  }
  void loop() {
    unsigned seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
      }
      drain();
      std::lock_guard<std::mutex> lk(mu_);
      if (--busy_ == 0) done_cv_.notify_one();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex job_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)> *task_ = nullptr;
  std::atomic<int> next_{0};
  int n_ = 0, busy_ = 0;
  unsigned gen_ = 0;
};

// valid cells (or faces) of every block: TreeData layout <-> compact
// fn(b0, b1) over block ranges; fields from 256 KB up are split over the
// host pool (the row copies of a 16M-cell field take tens of milliseconds
// on one core, a 0.4M-cell field a few hundred microseconds)
template <class F>
void for_blocks(int nblocks, size_t bytes, F &&fn) {
  HostPool &pool = HostPool::get();
  const int nt = bytes < (256u << 10) ? 1 : std::min(pool.size() * 2, std::max(1, nblocks / 16));
  if (nt <= 1) {
    fn(0, nblocks);
    return;
  }
  const int per = (nblocks + nt - 1) / nt;
  pool.run(nt, [&](int t) {
    const int b0 = t * per, b1 = std::min(nblocks, b0 + per);
    if (b0 < b1) fn(b0, b1);
  });
}

void pack(const Layout &L, int nblocks, const double *src, double *dst) {
  const int e[3] = {L.nb + (L.stag == 0), L.nd >= 2 ? L.nb + (L.stag == 1) : 1, L.nd == 3 ? L.nb + (L.stag == 2) : 1};
  const size_t per = (size_t)e[0] * e[1] * e[2];
  for_blocks(nblocks, nblocks * per * sizeof(double), [&](int b0, int b1) {
    size_t q = (size_t)b0 * per;
    for (int b = b0; b < b1; b++)
      for (int k = 0; k < e[2]; k++)
        for (int j = 0; j < e[1]; j++) {
          std::memcpy(dst + q, src + L.at(b, 0, j, k), e[0] * sizeof(double));
          q += e[0];
        }
  });
}
void unpack(const Layout &L, int nblocks, const double *src, double *dst) {
  const int e[3] = {L.nb + (L.stag == 0), L.nd >= 2 ? L.nb + (L.stag == 1) : 1, L.nd == 3 ? L.nb + (L.stag == 2) : 1};
  const size_t per = (size_t)e[0] * e[1] * e[2];
  for_blocks(nblocks, nblocks * per * sizeof(double), [&](int b0, int b1) {
    size_t q = (size_t)b0 * per;
    for (int b = b0; b < b1; b++)
      for (int k = 0; k < e[2]; k++)
        for (int j = 0; j < e[1]; j++) {
          std::memcpy(dst + L.at(b, 0, j, k), src + q, e[0] * sizeof(double));
          q += e[0];
        }
  });
}

int status_of(sayaka_mac *h) {
  if (!h->gpu) return SAYAKA_BAD_INPUT;
  if (!h->gpu->error().empty()) {
    h->err = h->gpu->error();
    return SAYAKA_CUDA_ERROR;
  }
  return SAYAKA_OK;
}

double *staging(sayaka_mac *h, size_t n) {
  if (h->pinned_n < n) {
    if (h->pinned) cudaFreeHost(h->pinned);
    h->pinned = nullptr;
    h->pinned_n = 0;
    if (cudaMallocHost(&h->pinned, n * sizeof(double)) != cudaSuccess) return nullptr;
    h->pinned_n = n;
  }
  return h->pinned;
}

// The calling thread's current device switched to `dev` for a scope and
// restored afterwards: a handle's calls run on the device its buffers live
// on, whatever device the caller has current.  Its own failures (no device)
// are not left pending as the thread's CUDA error.
struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int dev) {
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    if (cur == dev) return;
    if (cudaSetDevice(dev) == cudaSuccess)
      prev = cur;
    else
      cudaGetLastError();
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

template <typename F>
int guarded(sayaka_mac *h, F &&f) {
  if (!h) return SAYAKA_BAD_INPUT;
  if (!h->gpu) {
    h->err = "solver not created";
    return SAYAKA_BAD_INPUT;
  }
  DeviceScope on_device(h->gpu->device());
  try {
    const int r = f();
    if (r != SAYAKA_OK) return r;
  } catch (const std::exception &e) {
    h->err = e.what();
    return SAYAKA_BAD_INPUT;
  }
  return status_of(h);
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// tree mirror
int sayaka_tree_create(int32_t ndim, int32_t nb, int32_t min_level, int32_t max_level, int32_t capacity,
                       sayaka_tree **out) {
  if (!out || ndim < 2 || ndim > 3 || nb < 2 || (nb & 1) || min_level < 1 || max_level < min_level ||
      max_level > 16 || capacity < 1)
    return SAYAKA_BAD_INPUT;
  auto *h = new sayaka_tree;
  h->t.init(ndim, nb, min_level, max_level, capacity);
  *out = h;
  return SAYAKA_OK;
}
void sayaka_tree_destroy(sayaka_tree *t) { delete t; }

int sayaka_tree_init_uniform_root(sayaka_tree *t, const int32_t ndiv[3], const double lo[3], const double hi[3],
                                  const int32_t bc_type[6], const int32_t periodic[6]) {
  if (!t || !ndiv || !lo || !hi || !bc_type || !periodic) return SAYAKA_BAD_INPUT;
  long n = 1;
  for (int d = 0; d < 3; d++) {
    if (ndiv[d] < 1 || (d >= t->t.ndim && ndiv[d] != 1)) return SAYAKA_BAD_INPUT;
    n *= ndiv[d];
  }
  if (n > t->t.capacity) return SAYAKA_BAD_INPUT;
  for (int f = 0; f < 2 * t->t.ndim; f++)
    if (!periodic[f] && bc_type[f] > -20) return SAYAKA_BAD_INPUT;
  bool per[6];
  for (int f = 0; f < 6; f++) per[f] = periodic[f] != 0;
  t->t.init_uniform_root(ndiv, lo, hi, bc_type, per);
  t->dirty = true;
  return SAYAKA_OK;
}
int sayaka_tree_init_refine_to_min_level(sayaka_tree *t) {
  if (!t) return SAYAKA_BAD_INPUT;
  const int rc = t->t.init_refine_to_min_level();
  t->dirty = true;
  return rc ? SAYAKA_BAD_INPUT : SAYAKA_OK;
}
int sayaka_tree_set_refine_flags(sayaka_tree *t, const int32_t *flags, int32_t n) {
  if (!t || !flags || n < 0 || n > t->t.capacity) return SAYAKA_BAD_INPUT;
  for (int i = 0; i < n; i++) t->t.refine_flag[i] = flags[i];
  return SAYAKA_OK;
}
int sayaka_tree_set_coarsen_flags(sayaka_tree *t, const int32_t *flags, int32_t n) {
  if (!t || !flags || n < 0 || n > t->t.capacity) return SAYAKA_BAD_INPUT;
  for (int i = 0; i < n; i++) t->t.coarsen_flag[i] = flags[i];
  return SAYAKA_OK;
}
int sayaka_tree_regrid(sayaka_tree *t) {
  if (!t) return SAYAKA_BAD_INPUT;
  const int rc = t->t.regrid();
  t->dirty = true;
  return rc ? SAYAKA_BAD_INPUT : SAYAKA_OK;
}
int32_t sayaka_tree_num_blocks(const sayaka_tree *t) { return t ? t->t.num_blocks : -1; }

int sayaka_tree_get_tables(sayaka_tree *t, sayaka_tree_tables *o) {
  if (!t || !o) return SAYAKA_BAD_INPUT;
  refresh(t);
  o->ndim = t->t.ndim;
  o->nb = t->t.nb;
  o->num_blocks = t->t.num_blocks;
  o->min_level = t->t.min_level;
  o->max_level = t->t.max_level;
  o->level = t->level.data();
  o->neighbor = t->neighbor.data();
  o->child = t->child.data();
  o->parent = t->parent.data();
  o->which_child = t->wc.data();
  o->node_type = t->nt.data();
  o->block_len = t->len.data();
  return SAYAKA_OK;
}
int sayaka_tree_get_geometry(const sayaka_tree *t, double *lo, double *hi, double *center) {
  if (!t) return SAYAKA_BAD_INPUT;
  for (int b = 0; b < t->t.num_blocks; b++)
    for (int d = 0; d < 3; d++) {
      if (lo) lo[b * 3 + d] = t->t.nodes[b].lo[d];
      if (hi) hi[b * 3 + d] = t->t.nodes[b].hi[d];
      if (center) center[b * 3 + d] = t->t.nodes[b].center[d];
    }
  return SAYAKA_OK;
}
int sayaka_tree_get_node_type2(const sayaka_tree *t, int32_t *out) {
  if (!t || !out) return SAYAKA_BAD_INPUT;
  for (int b = 0; b < t->t.num_blocks; b++)
    for (int f = 0; f < 6; f++) out[b * 6 + f] = t->t.nodes[b].node_type2[f];
  return SAYAKA_OK;
}
int sayaka_tree_get_surrounding(const sayaka_tree *t, int32_t *blocks, int32_t *types, int32_t *bcrefs) {
  if (!t) return SAYAKA_BAD_INPUT;
  for (int b = 0; b < t->t.num_blocks; b++)
    for (int s = 0; s < 27; s++) {
      if (blocks) blocks[b * 27 + s] = t->t.surr[b].blocks[s];
      if (types) types[b * 27 + s] = t->t.surr[b].types[s];
      if (bcrefs) bcrefs[b * 27 + s] = t->t.surr[b].bcrefs[s];
    }
  return SAYAKA_OK;
}
int sayaka_tree_get_tower(const sayaka_tree *tc, int32_t L, int32_t *blocks, int32_t *n, int32_t *begin_end) {
  sayaka_tree *t = const_cast<sayaka_tree *>(tc);
  if (!t || L < 1 || L > t->t.max_level || !n) return SAYAKA_BAD_INPUT;
  refresh(t);
  const Tower &tw = t->towers[L];
  *n = (int)tw.blocks.size();
  if (blocks) std::memcpy(blocks, tw.blocks.data(), tw.blocks.size() * sizeof(int32_t));
  if (begin_end)
    for (int l = 1; l <= L; l++) {
      begin_end[2 * (l - 1)] = tw.empty() ? 0 : tw.begin[l];
      begin_end[2 * (l - 1) + 1] = tw.empty() ? 0 : tw.end[l];
    }
  return SAYAKA_OK;
}
int sayaka_tree_get_face_regs(const sayaka_tree *tc, int32_t L, int32_t *regs) {
  sayaka_tree *t = const_cast<sayaka_tree *>(tc);
  if (!t || L < 1 || L > t->t.max_level || !regs) return SAYAKA_BAD_INPUT;
  refresh(t);
  const Tower &tw = t->towers[L];
  const int nf = t->t.num_face();
  size_t q = 0;
  for (size_t p = 0; p < tw.blocks.size(); p++)
    for (int f = 0; f < nf; f++) {
      const FaceReg &r = tw.regs[p * 6 + f];
      regs[q++] = r.type;
      regs[q++] = r.neigh;
      for (int d = 0; d < 3; d++) regs[q++] = r.type == kFaceFineCrse ? r.fc_off[d] : 0;
      for (int c = 0; c < 4; c++) regs[q++] = r.type == kFaceCrseFine ? r.cf_neigh[c] : -1;
    }
  return SAYAKA_OK;
}

// ---------------------------------------------------------------------------
// solver
void sayaka_params_default(sayaka_params *p) {
  if (!p) return;
  SolverParams d;
  p->max_iter = d.max_iter;
  p->tol_rel = d.tol_rel;
  p->tol_abs = d.tol_abs;
  p->n_post_smooth = d.n_post;
  p->use_mg_precond = d.use_mg_precond;
  p->bot_tol_rel = d.bot_tol_rel;
  p->bot_tol_abs = d.bot_tol_abs;
  p->bot_max_iter = d.bot_max_iter;
  p->precision = d.precision;
  p->bottom = d.bottom;
  p->verbose = d.verbose;
  p->graph = d.graph;
  p->vcycle_kernel = d.vcycle_kernel;
  p->pdl = d.pdl;
  p->cluster_cells = d.cluster_cells;
  p->smooth_variant = d.smooth_variant;
  p->learned = d.learned;
  p->bottom_level = d.bottom_level;
  p->bottom_half = d.bottom_half;
  p->sublevel_order = d.sublevel_order;
  p->smoother = d.smoother;
  p->inner_sweeps = d.inner_sweeps;
  p->per_problem = d.per_problem;
  p->uniform = d.uniform;
  p->bottom_refresh = d.bottom_refresh;
  p->learned_tc05 = d.learned_tc05;
  p->learned_loss = d.learned_loss;
  p->prolong_form = d.prolong_form;
  p->vcycle_out = d.vcycle_out;
  p->relax_omega = d.relax_omega;
}

int sayaka_mac_create(const sayaka_tree_tables *tb, sayaka_mac **out) {
  if (!tb || !out) return SAYAKA_BAD_INPUT;
  *out = nullptr;
  const int n = tb->num_blocks;
  if (n <= 0 || tb->ndim < 2 || tb->ndim > 3 || tb->nb < 2 || (tb->nb & 1) || tb->min_level < 1 ||
      tb->max_level < tb->min_level || !tb->level || !tb->neighbor || !tb->child || !tb->parent ||
      !tb->which_child || !tb->node_type || !tb->block_len)
    return SAYAKA_BAD_INPUT;
  TreeTables tt;
  tt.ndim = tb->ndim;
  tt.nb = tb->nb;
  tt.num_blocks = n;
  tt.min_level = tb->min_level;
  tt.max_level = tb->max_level;
  tt.level.assign(tb->level, tb->level + n);
  tt.neighbor.assign(tb->neighbor, tb->neighbor + (size_t)n * 6);
  tt.child.assign(tb->child, tb->child + (size_t)n * 8);
  tt.parent.assign(tb->parent, tb->parent + n);
  tt.which_child.assign(tb->which_child, tb->which_child + n);
  tt.node_type.assign(tb->node_type, tb->node_type + n);
  tt.block_len.assign(tb->block_len, tb->block_len + (size_t)n * 3);
  // table sanity: ids in range, levels in range
  for (int b = 0; b < n; b++) {
    if (tt.level[b] < 1 || tt.level[b] > tt.max_level) return SAYAKA_BAD_INPUT;
    for (int f = 0; f < 6; f++)
      if (tt.neighbor[b * 6 + f] >= n) return SAYAKA_BAD_INPUT;
    for (int c = 0; c < 8; c++)
      if (tt.child[b * 8 + c] >= n) return SAYAKA_BAD_INPUT;
    if (tt.parent[b] >= n) return SAYAKA_BAD_INPUT;
  }
  auto *h = new sayaka_mac;
  try {
    h->gpu.reset(new MacGpu(tt));
  } catch (const std::exception &e) {
    h->err = e.what();
  }
  if (!h->gpu || !h->gpu->error().empty()) {
    const int st = SAYAKA_CUDA_ERROR;
    delete h;
    return st;
  }
  *out = h;
  return SAYAKA_OK;
}

void sayaka_mac_destroy(sayaka_mac *h) {
  if (h && h->gpu) {
    DeviceScope on_device(h->gpu->device());
    delete h;
    return;
  }
  delete h;
}

const char *sayaka_mac_last_error(const sayaka_mac *h) {
  if (!h) return "null handle";
  if (!h->err.empty()) return h->err.c_str();
  if (h->gpu && !h->gpu->error().empty()) return h->gpu->error().c_str();
  return "";
}

int sayaka_mac_set_scalars(sayaka_mac *h, double alpha, double beta) {
  return guarded(h, [&] {
    h->gpu->set_scalars(alpha, beta);
    return SAYAKA_OK;
  });
}

int sayaka_mac_set_coef_b(sayaka_mac *h, int32_t dir, const double *face, int32_t ncomp, int32_t ngrow,
                          int32_t comp) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (dir < 0 || dir >= g.ndim() || !face) return (int)SAYAKA_BAD_INPUT;
    Layout L(g.ndim(), g.nb(), ncomp, ngrow, comp, dir);
    if (!L.ok()) return (int)SAYAKA_BAD_INPUT;
    std::vector<double> c((size_t)g.num_blocks() * g.nfb());
    pack(L, g.num_blocks(), face, c.data());
    g.set_coef_b_leaf(dir, c.data());
    return (int)SAYAKA_OK;
  });
}

int sayaka_mac_set_ib_frac_by_ls(sayaka_mac *h, const double *ls, int32_t ncomp, int32_t ngrow, int32_t comp) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (!ls || ngrow < 1) return (int)SAYAKA_BAD_INPUT;
    Layout L(g.ndim(), g.nb(), ncomp, ngrow, comp, -1);
    if (!L.ok()) return (int)SAYAKA_BAD_INPUT;
    if (ncomp == 1) {  // the buffer is the grown boxes already
      g.set_ib_frac_by_ls(ls, ngrow);
      return (int)SAYAKA_OK;
    }
    // extract the grown box of component `comp` for every block
    std::vector<double> grown((size_t)g.num_blocks() * L.cap);
    for (int b = 0; b < g.num_blocks(); b++)
      std::memcpy(&grown[(size_t)b * L.cap], ls + (size_t)b * L.cap * ncomp + (size_t)comp * L.cap,
                  L.cap * sizeof(double));
    g.set_ib_frac_by_ls(grown.data(), ngrow);
    return (int)SAYAKA_OK;
  });
}

int sayaka_mac_set_ib_frac_by_ls_compact(sayaka_mac *h, const double *ls, int32_t ngrow, int32_t on_device) {
  return guarded(h, [&] {
    if (!ls || ngrow < 1 || ngrow > 8) return (int)SAYAKA_BAD_INPUT;
    h->gpu->set_ib_frac_by_ls(ls, ngrow, on_device != 0);
    return (int)SAYAKA_OK;
  });
}

int sayaka_mac_set_ib_frac_compact(sayaka_mac *h, const double *vol, const double *a0, const double *a1,
                                   const double *a2) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (!vol || !a0 || (g.ndim() >= 2 && !a1) || (g.ndim() == 3 && !a2)) return (int)SAYAKA_BAD_INPUT;
    const double *a[3] = {a0, a1, a2};
    g.set_ib_frac_leaf(vol, a);
    return (int)SAYAKA_OK;
  });
}

int sayaka_mac_set_bc(sayaka_mac *h, const int32_t *bc) {
  return guarded(h, [&] {
    if (!bc) return (int)SAYAKA_BAD_INPUT;
    for (int i = 0; i < h->gpu->num_blocks() * 6; i++)
      if (bc[i] < -1 || bc[i] > 2) return (int)SAYAKA_BAD_INPUT;
    h->gpu->set_bc_types(bc);
    return (int)SAYAKA_OK;
  });
}

int sayaka_mac_fix_bc(sayaka_mac *h, const double *phi, int32_t pn, int32_t pg, int32_t pc, double *rhs, int32_t rn,
                      int32_t rg, int32_t rc) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (!phi || !rhs || pg < 1) return (int)SAYAKA_BAD_INPUT;
    Layout P(g.ndim(), g.nb(), pn, pg, pc, -1), R(g.ndim(), g.nb(), rn, rg, rc, -1);
    if (!P.ok() || !R.ok()) return (int)SAYAKA_BAD_INPUT;
    std::vector<double> grown((size_t)g.num_blocks() * P.cap);
    for (int b = 0; b < g.num_blocks(); b++)
      std::memcpy(&grown[(size_t)b * P.cap], phi + (size_t)b * P.cap * pn + (size_t)pc * P.cap,
                  P.cap * sizeof(double));
    std::vector<double> r((size_t)g.num_blocks() * g.ncell());
    pack(R, g.num_blocks(), rhs, r.data());
    g.fix_bc(grown.data(), pg, r.data());
    unpack(R, g.num_blocks(), r.data(), rhs);
    return (int)SAYAKA_OK;
  });
}

// the device address of `p` when it is pinned (page-locked) host memory the
// GPU can read and write directly, else null (pageable memory is never
// touched by a kernel: it goes through the staging copy)
static const void *pinned_device_ptr(const void *p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

static int set_field(sayaka_mac *h, const double *data, int32_t ncomp, int32_t ngrow, int32_t comp, bool rhs) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (!data) return (int)SAYAKA_BAD_INPUT;
    Layout L(g.ndim(), g.nb(), ncomp, ngrow, comp, -1);
    if (!L.ok()) return (int)SAYAKA_BAD_INPUT;
    // pinned TreeData: gathered by the GPU straight from host memory
    if (const void *dp = pinned_device_ptr(data)) {
      if (g.set_field_td(static_cast<const double *>(dp), ncomp, ngrow, comp, rhs) != 0) return status_of(h);
      return (int)SAYAKA_OK;
    }
    double *st = staging(h, (size_t)g.num_blocks() * g.ncell());
    if (!st) return (int)SAYAKA_CUDA_ERROR;
    pack(L, g.num_blocks(), data, st);
    if (rhs)
      g.set_rhs(st);
    else
      g.set_sol(st);
    cudaStreamSynchronize(g.stream());
    return (int)SAYAKA_OK;
  });
}

int sayaka_mac_set_rhs(sayaka_mac *h, const double *d, int32_t nc, int32_t ng, int32_t c) {
  return set_field(h, d, nc, ng, c, true);
}
int sayaka_mac_set_init_sol(sayaka_mac *h, const double *d, int32_t nc, int32_t ng, int32_t c) {
  return set_field(h, d, nc, ng, c, false);
}
int sayaka_mac_set_zero_sol(sayaka_mac *h) {
  return guarded(h, [&] {
    h->gpu->zero_sol();
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_get_sol(sayaka_mac *h, double *data, int32_t ncomp, int32_t ngrow, int32_t comp) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (!data) return (int)SAYAKA_BAD_INPUT;
    Layout L(g.ndim(), g.nb(), ncomp, ngrow, comp, -1);
    if (!L.ok()) return (int)SAYAKA_BAD_INPUT;
    // pinned TreeData: scattered by the GPU straight into host memory
    if (const void *dp = pinned_device_ptr(data)) {
      if (g.get_sol_td(static_cast<double *>(const_cast<void *>(dp)), ncomp, ngrow, comp) != 0) return status_of(h);
      return (int)SAYAKA_OK;
    }
    double *st = staging(h, (size_t)g.num_blocks() * g.ncell());
    if (!st) return (int)SAYAKA_CUDA_ERROR;
    g.get_sol(st);
    if (!g.error().empty()) return status_of(h);  // the copy failed: leave the caller's buffer alone
    unpack(L, g.num_blocks(), st, data);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_set_rhs_compact(sayaka_mac *h, const double *cells, int32_t on_device) {
  return guarded(h, [&] {
    if (!cells) return (int)SAYAKA_BAD_INPUT;
    h->gpu->set_rhs(cells, on_device != 0);
    cudaStreamSynchronize(h->gpu->stream());
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_get_sol_compact(sayaka_mac *h, double *cells, int32_t on_device) {
  return guarded(h, [&] {
    if (!cells) return (int)SAYAKA_BAD_INPUT;
    h->gpu->get_sol(cells, on_device != 0);
    return (int)SAYAKA_OK;
  });
}

int sayaka_mac_set_params(sayaka_mac *h, const sayaka_params *p) {
  return guarded(h, [&] {
    if (!p || p->max_iter < 0 || p->n_post_smooth < 0 || p->bot_max_iter < 0 || p->precision < 0 ||
        p->precision > 1 || p->bottom < 0 || p->bottom > 1)
      return (int)SAYAKA_BAD_INPUT;
    SolverParams s;
    s.max_iter = p->max_iter;
    s.tol_rel = p->tol_rel;
    s.tol_abs = p->tol_abs;
    s.n_post = p->n_post_smooth;
    s.use_mg_precond = p->use_mg_precond;
    s.bot_tol_rel = p->bot_tol_rel;
    s.bot_tol_abs = p->bot_tol_abs;
    s.bot_max_iter = p->bot_max_iter;
    s.precision = p->precision;
    s.bottom = p->bottom;
    s.verbose = p->verbose;
    s.graph = p->graph;
    s.vcycle_kernel = p->vcycle_kernel;
    s.pdl = p->pdl;
    s.cluster_cells = p->cluster_cells;
    s.smooth_variant = p->smooth_variant;
    s.learned = p->learned;
    s.bottom_level = p->bottom_level;
    s.bottom_half = p->bottom_half;
    s.sublevel_order = p->sublevel_order;
    if (p->smoother < 0 || p->smoother > 1 || p->inner_sweeps < 1 || p->inner_sweeps > 64)
      return (int)SAYAKA_BAD_INPUT;
    s.smoother = p->smoother;
    s.inner_sweeps = p->inner_sweeps;
    if (p->per_problem < 0 || p->per_problem > 1) return (int)SAYAKA_BAD_INPUT;
    s.per_problem = p->per_problem;
    if (p->uniform < 0 || p->uniform > 1) return (int)SAYAKA_BAD_INPUT;
    s.uniform = p->uniform;
    if (p->bottom_refresh < 0 || p->bottom_refresh > 1) return (int)SAYAKA_BAD_INPUT;
    s.bottom_refresh = p->bottom_refresh;
    if (p->learned_tc05 < 0 || p->learned_tc05 > 1) return (int)SAYAKA_BAD_INPUT;
    s.learned_tc05 = p->learned_tc05;
    if (p->learned_loss < 0 || p->learned_loss > 1) return (int)SAYAKA_BAD_INPUT;
    s.learned_loss = p->learned_loss;
    if (p->prolong_form < 0 || p->prolong_form > 1) return (int)SAYAKA_BAD_INPUT;
    s.prolong_form = p->prolong_form;
    if (p->vcycle_out < 0 || p->vcycle_out > 3) return (int)SAYAKA_BAD_INPUT;
    s.vcycle_out = p->vcycle_out;
    if (!(p->relax_omega > 0.0 && p->relax_omega < 2.0)) return (int)SAYAKA_BAD_INPUT;
    s.relax_omega = p->relax_omega;
    h->gpu->set_params(s);
    return (int)SAYAKA_OK;
  });
}

static int solve_with(sayaka_mac *h, sayaka_solve_info *info, int (MacGpu::*fn)(SolveInfo *)) {
  return guarded(h, [&] {
    SolveInfo si;
    const int st = (h->gpu.get()->*fn)(&si);
    if (info) {
      info->status = si.status;
      info->iterations = si.iterations;
      info->rnorm0 = si.rnorm0;
      info->rnorm = si.rnorm;
      info->seconds = si.seconds;
    }
    if (st < 0) return (int)SAYAKA_CUDA_ERROR;
    return si.status == 0 ? (int)SAYAKA_OK : (si.status == 1 ? (int)SAYAKA_BREAKDOWN : (int)SAYAKA_NOT_CONVERGED);
  });
}
int sayaka_mac_mg_solve(sayaka_mac *h, sayaka_solve_info *info) { return solve_with(h, info, &MacGpu::mg_solve); }
int sayaka_mac_relax_solve(sayaka_mac *h, sayaka_solve_info *info) {
  return solve_with(h, info, &MacGpu::relax_solve);
}
int sayaka_mac_cg_solve(sayaka_mac *h, sayaka_solve_info *info) {
  return guarded(h, [&] {
    SolveInfo si;
    const int st = h->gpu->cg_solve(&si);
    if (info) {
      info->status = si.status;
      info->iterations = si.iterations;
      info->rnorm0 = si.rnorm0;
      info->rnorm = si.rnorm;
      info->seconds = si.seconds;
    }
    if (st < 0) return (int)SAYAKA_CUDA_ERROR;
    return si.status == 0 ? (int)SAYAKA_OK : (si.status == 1 ? (int)SAYAKA_BREAKDOWN : (int)SAYAKA_NOT_CONVERGED);
  });
}

int sayaka_mac_prepare(sayaka_mac *h) {
  return guarded(h, [&] {
    if (h->gpu->params().bottom != 1 || !h->gpu->params().use_mg_precond) {
      h->err = "prepare needs params.bottom = 1 and use_mg_precond = 1";
      return (int)SAYAKA_BAD_INPUT;
    }
    return h->gpu->prepare_device() == 0 ? (int)SAYAKA_OK : (int)SAYAKA_CUDA_ERROR;
  });
}
int sayaka_mac_cg_solve_async(sayaka_mac *h) {
  return guarded(h, [&] { return h->gpu->cg_solve_enqueue() == 0 ? (int)SAYAKA_OK : (int)SAYAKA_BAD_INPUT; });
}
int sayaka_mac_solve_info(sayaka_mac *h, sayaka_solve_info *info) {
  return guarded(h, [&] {
    SolveInfo si;
    if (h->gpu->solve_state(&si) != 0) return (int)SAYAKA_CUDA_ERROR;
    if (info) {
      info->status = si.status;
      info->iterations = si.iterations;
      info->rnorm0 = si.rnorm0;
      info->rnorm = si.rnorm;
      info->seconds = 0;
    }
    return (int)SAYAKA_OK;
  });
}
void *sayaka_mac_stream(sayaka_mac *h) { return (h && h->gpu) ? (void *)h->gpu->stream() : nullptr; }
int sayaka_mac_enqueue_kernel(sayaka_mac *h, int32_t which, int32_t L) {
  return guarded(h, [&] { return h->gpu->enqueue_kernel(which, L) == 0 ? (int)SAYAKA_OK : (int)SAYAKA_BAD_INPUT; });
}
int sayaka_mac_launch_counts(sayaka_mac *h, int32_t *pro, int32_t *per, int32_t *epi) {
  return guarded(h, [&] {
    if (pro) *pro = MacGpu::kPrologueKernels;
    if (per) *per = h->gpu->kernels_per_iteration();
    if (epi) *epi = MacGpu::kEpilogueKernels;
    return (int)SAYAKA_OK;
  });
}
int32_t sayaka_mac_tower_size(sayaka_mac *h, int32_t L, int32_t sublevel) {
  return (h && h->gpu) ? h->gpu->tower_size(L, sublevel) : -1;
}

int sayaka_mac_flux(sayaka_mac *h, int32_t dir, const double *phi, int32_t pn, int32_t pg, int32_t pc, double *flux,
                    int32_t fn, int32_t fg, int32_t fc) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (dir < 0 || dir >= g.ndim() || !phi || !flux) return (int)SAYAKA_BAD_INPUT;
    Layout P(g.ndim(), g.nb(), pn, pg, pc, -1), F(g.ndim(), g.nb(), fn, fg, fc, dir);
    if (!P.ok() || !F.ok()) return (int)SAYAKA_BAD_INPUT;
    std::vector<double> p((size_t)g.num_blocks() * g.ncell()), f((size_t)g.num_blocks() * g.nfb());
    pack(P, g.num_blocks(), phi, p.data());
    g.flux(dir, p.data(), f.data());
    // leaf blocks only (the tower the flux is defined on)
    std::vector<double> full((size_t)g.num_blocks() * g.nfb());
    pack(F, g.num_blocks(), flux, full.data());
    for (int b : g.tower_blocks(g.finest()))
      std::memcpy(&full[(size_t)b * g.nfb()], &f[(size_t)b * g.nfb()], g.nfb() * sizeof(double));
    unpack(F, g.num_blocks(), full.data(), flux);
    return (int)SAYAKA_OK;
  });
}

// ---- learned block correction ----
int32_t sayaka_mac_learned_nparam(void) { return learned::kNParam; }
int sayaka_mac_learned_collect(sayaka_mac *h, int32_t max_iter, int32_t *iterates) {
  return sayaka_mac_learned_collect_sampled(h, max_iter, 0, iterates);
}
int sayaka_mac_learned_collect_sampled(sayaka_mac *h, int32_t max_iter, int32_t max_samples, int32_t *iterates) {
  return guarded(h, [&] {
    if (!h->gpu->learned_supported()) {
      h->err = "learned correction: 2D trees with 8x8 or 16x16 blocks only";
      return (int)SAYAKA_BAD_INPUT;
    }
    if (max_samples < 0) return (int)SAYAKA_BAD_INPUT;
    const int n = h->gpu->learned_collect(max_iter > 0 ? max_iter : 200, max_samples);
    if (iterates) *iterates = n < 0 ? 0 : n;
    return n < 0 ? (int)SAYAKA_CUDA_ERROR : (int)SAYAKA_OK;
  });
}
int sayaka_mac_learned_train(sayaka_mac *h, int32_t epochs, float lr, int32_t batch, uint32_t seed, float *loss) {
  return guarded(h, [&] {
    if (epochs < 0 || batch < 1 || !(lr > 0)) return (int)SAYAKA_BAD_INPUT;
    if (h->gpu->learned_samples() == 0) {
      h->err = "learned correction: no training pairs (call sayaka_mac_learned_collect first)";
      return (int)SAYAKA_BAD_INPUT;
    }
    const float l = h->gpu->learned_train(epochs, lr, batch, seed);
    if (loss) *loss = l;
    return l < 0 ? (int)SAYAKA_CUDA_ERROR : (int)SAYAKA_OK;
  });
}
int sayaka_mac_learned_eval(sayaka_mac *h, float *loss) {
  return guarded(h, [&] {
    if (h->gpu->learned_samples() == 0) {
      h->err = "learned correction: no pairs to evaluate (call sayaka_mac_learned_collect first)";
      return (int)SAYAKA_BAD_INPUT;
    }
    const float l = h->gpu->learned_eval();
    if (loss) *loss = l;
    return l < 0 ? (int)SAYAKA_CUDA_ERROR : (int)SAYAKA_OK;
  });
}
int sayaka_mac_learned_get_weights(sayaka_mac *h, float *w, int32_t n) {
  return guarded(h, [&] { return h->gpu->learned_get_weights(w, n) == 0 ? (int)SAYAKA_OK : (int)SAYAKA_BAD_INPUT; });
}
int sayaka_mac_learned_set_weights(sayaka_mac *h, const float *w, int32_t n) {
  return guarded(h, [&] {
    if (!w || n != learned::kNParam || !h->gpu->learned_supported()) return (int)SAYAKA_BAD_INPUT;
    return h->gpu->learned_set_weights(w, n) == 0 ? (int)SAYAKA_OK : (int)SAYAKA_CUDA_ERROR;
  });
}
int sayaka_mac_learned_loss_grad(sayaka_mac *h, const float *feat, const float *aux, int32_t n, float *grad,
                                 float *loss) {
  return guarded(h, [&] {
    if (!feat || !aux || !grad || n < 1 || !h->gpu->learned_supported()) return (int)SAYAKA_BAD_INPUT;
    const float l = h->gpu->learned_loss_grad(feat, aux, n, grad);
    if (loss) *loss = l;
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_learned_forward(sayaka_mac *h, const float *feat, int32_t n, float *y) {
  return guarded(h, [&] {
    if (!feat || !y || n < 1 || !h->gpu->learned_supported()) return (int)SAYAKA_BAD_INPUT;
    return h->gpu->learned_forward(feat, n, y) == 0 ? (int)SAYAKA_OK : (int)SAYAKA_CUDA_ERROR;
  });
}

// ---- projection step around the solve ----
int sayaka_mac_set_rhs_div(sayaka_mac *h, const double *const *u, int32_t ncomp, int32_t ngrow, int32_t ucomp,
                           int32_t wcomp, double scale) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (!u) return (int)SAYAKA_BAD_INPUT;
    const size_t nf = (size_t)g.num_blocks() * g.nfb();
    std::vector<std::vector<double>> uc(g.ndim()), wc(g.ndim());
    const double *up[3] = {}, *wp[3] = {};
    for (int d = 0; d < g.ndim(); d++) {
      if (!u[d]) return (int)SAYAKA_BAD_INPUT;
      Layout Lu(g.ndim(), g.nb(), ncomp, ngrow, ucomp, d);
      if (!Lu.ok()) return (int)SAYAKA_BAD_INPUT;
      uc[d].resize(nf);
      pack(Lu, g.num_blocks(), u[d], uc[d].data());
      up[d] = uc[d].data();
      if (wcomp >= 0) {
        Layout Lw(g.ndim(), g.nb(), ncomp, ngrow, wcomp, d);
        if (!Lw.ok()) return (int)SAYAKA_BAD_INPUT;
        wc[d].resize(nf);
        pack(Lw, g.num_blocks(), u[d], wc[d].data());
        wp[d] = wc[d].data();
      }
    }
    g.rhs_from_div(up, wcomp >= 0 ? wp : nullptr, scale);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_correct_vel(sayaka_mac *h, int32_t dir, double dt, double *u, int32_t ncomp, int32_t ngrow,
                           int32_t comp) {
  return guarded(h, [&] {
    MacGpu &g = *h->gpu;
    if (dir < 0 || dir >= g.ndim() || !u) return (int)SAYAKA_BAD_INPUT;
    Layout L(g.ndim(), g.nb(), ncomp, ngrow, comp, dir);
    if (!L.ok()) return (int)SAYAKA_BAD_INPUT;
    std::vector<double> c((size_t)g.num_blocks() * g.nfb());
    pack(L, g.num_blocks(), u, c.data());
    g.correct_vel(dir, dt, c.data());
    unpack(L, g.num_blocks(), c.data(), u);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_init_from(sayaka_mac *h, const sayaka_mac *old) {
  return guarded(h, [&] {
    if (!old || !old->gpu) return (int)SAYAKA_BAD_INPUT;
    std::string why;
    const int st = h->gpu->init_solution_from(*old->gpu, &why);
    if (st == 1) {
      h->err = why;
      return (int)SAYAKA_BAD_INPUT;
    }
    return st == 0 ? (int)SAYAKA_OK : (int)SAYAKA_CUDA_ERROR;
  });
}
int sayaka_mac_init_new_block_data(sayaka_mac *h, const sayaka_mac *old, const double *bc_val) {
  return guarded(h, [&] {
    if (!old || !old->gpu) return (int)SAYAKA_BAD_INPUT;
    std::string why;
    const int st = h->gpu->init_new_block_data(*old->gpu, bc_val, &why);
    if (st == 1) {
      h->err = why;
      return (int)SAYAKA_BAD_INPUT;
    }
    if (st != 0 && !why.empty()) h->err = why;
    return st == 0 ? (int)SAYAKA_OK : (int)SAYAKA_CUDA_ERROR;
  });
}
int32_t sayaka_cuda_peek_error(void) { return (int32_t)cudaPeekAtLastError(); }
int sayaka_fp_selftest(const double *d, const float *f, int n, float *narrow, float *narrow_hw, double *widen,
                       double *widen_hw, double *widen0, double *widen0_hw) {
  if (n < 0 || (n > 0 && (!d || !f || !narrow || !narrow_hw || !widen || !widen_hw || !widen0 || !widen0_hw)))
    return SAYAKA_BAD_INPUT;
  return sayaka_gb300::fp_selftest(d, f, n, narrow, narrow_hw, widen, widen_hw, widen0, widen0_hw) == 0
             ? SAYAKA_OK
             : SAYAKA_CUDA_ERROR;
}
int sayaka_mac_get_rhs_compact(sayaka_mac *h, double *out) {
  return guarded(h, [&] {
    if (!out) return (int)SAYAKA_BAD_INPUT;
    h->gpu->get_rhs(out);
    return (int)SAYAKA_OK;
  });
}

// ---- parity hooks ----
int sayaka_mac_apply_compact(sayaka_mac *h, int32_t L, const double *x, double *y) {
  return guarded(h, [&] {
    if (L < 1 || !x || !y) return (int)SAYAKA_BAD_INPUT;
    h->gpu->apply(L, x, y);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_residual_compact(sayaka_mac *h, int32_t L, const double *x, const double *rhs, double *r) {
  return guarded(h, [&] {
    if (L < 1 || !x || !rhs || !r) return (int)SAYAKA_BAD_INPUT;
    h->gpu->residual(L, x, rhs, r);
    return (int)SAYAKA_OK;
  });
}
int32_t sayaka_mac_problem_count(const sayaka_mac *h) {
  if (!h || !h->gpu) return -1;
  return h->gpu->problems();
}
int32_t sayaka_mac_problem_states(sayaka_mac *h, int32_t *iterations, double *rel_resid, int32_t n) {
  if (!h || !h->gpu || n < 0) return -1;
  DeviceScope on_device(h->gpu->device());
  std::vector<int> it(std::max(0, n));
  const int r = h->gpu->problem_states(it.data(), rel_resid, n);
  if (r >= 0 && iterations)
    for (int k = 0; k < n && k < r; k++) iterations[k] = it[k];
  return r;
}
int32_t sayaka_mac_uniform_blocks(sayaka_mac *h) {
  if (!h || !h->gpu) return -1;
  int n = -1;
  const int rc = guarded(h, [&] {
    n = h->gpu->uniform_blocks();
    return n < 0 ? (int)SAYAKA_CUDA_ERROR : (int)SAYAKA_OK;
  });
  return rc == (int)SAYAKA_OK ? n : -1;
}
int32_t sayaka_mac_bottom_level(const sayaka_mac *h) {
  if (!h || !h->gpu) return -1;
  return h->gpu->bottom_level();
}
int32_t sayaka_smoother_variants(void) { return kRbgsVariants; }
int32_t sayaka_mac_tuned_smoother(sayaka_mac *h, int32_t precision, float *us, int32_t n) {
  if (!h || !h->gpu) return -1;
  float tmp[16] = {};
  const int v = h->gpu->tuned_smoother(precision, tmp, 16);
  if (us)
    for (int i = 0; i < n && i < 16; i++) us[i] = tmp[i];
  return v;
}
int sayaka_mac_residual_norm_noalloc(sayaka_mac *h, int32_t L, const double *x, const double *rhs, double *r,
                                     double *norms, void *stream) {
  if (!h) return SAYAKA_BAD_INPUT;
  if (!h->gpu) {
    h->err = "solver not created";
    return SAYAKA_BAD_INPUT;
  }
  // the handle's device is current for the scratch lookup and the launch,
  // whatever device the caller has current (restored on return)
  DeviceScope on_device(h->gpu->device());
  std::string why;
  const cudaStream_t s = stream ? (cudaStream_t)stream : h->gpu->stream();
  const int st = h->gpu->residual_norm_noalloc(L, x, rhs, r, norms, s, &why);
  if (st == 0) return SAYAKA_OK;
  h->err = why;
  return st == 1 ? SAYAKA_BAD_INPUT : SAYAKA_CUDA_ERROR;
}
int sayaka_mac_device_kernel_compact(sayaka_mac *h, int32_t which, int32_t L, int32_t variant, const double *in,
                                     const double *in2, double *out) {
  return guarded(h, [&] {
    const int r = h->gpu->device_kernel_compact(which, L, variant, in, in2, out);
    if (r == 1) {
      h->err = "device_kernel_compact: which must be 0..3, L a tower of the tree (which 1, 2), a smoother variant "
               "(which 1) or 1..1024 (which 2), pointers non-null";
      return (int)SAYAKA_BAD_INPUT;
    }
    return (int)SAYAKA_OK;  // CUDA errors are reported by status_of
  });
}
int sayaka_mac_smooth_compact(sayaka_mac *h, int32_t L, const double *phi, const double *rhs, double *out) {
  return guarded(h, [&] {
    if (L < 1 || !phi || !rhs || !out) return (int)SAYAKA_BAD_INPUT;
    h->gpu->smooth(L, phi, rhs, out);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_restrict_compact(sayaka_mac *h, const double *in, double *out) {
  return guarded(h, [&] {
    if (!in || !out) return (int)SAYAKA_BAD_INPUT;
    h->gpu->restrict_sweep(in, out);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_prolong_compact(sayaka_mac *h, const double *in, double *out) {
  return guarded(h, [&] {
    if (!in || !out) return (int)SAYAKA_BAD_INPUT;
    h->gpu->prolong_sweep(in, out);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_vcycle_compact(sayaka_mac *h, const double *p, double *phat) {
  return guarded(h, [&] {
    if (!p || !phat) return (int)SAYAKA_BAD_INPUT;
    h->gpu->vcycle(p, phat);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_flux_compact(sayaka_mac *h, int32_t dir, const double *phi, double *flux) {
  return guarded(h, [&] {
    if (dir < 0 || dir >= h->gpu->ndim() || !phi || !flux) return (int)SAYAKA_BAD_INPUT;
    h->gpu->flux(dir, phi, flux);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_fix_bc_compact(sayaka_mac *h, const double *phi_grown, int32_t ngrow, double *rhs) {
  return guarded(h, [&] {
    if (!phi_grown || !rhs || ngrow < 1) return (int)SAYAKA_BAD_INPUT;
    h->gpu->fix_bc(phi_grown, ngrow, rhs);
    return (int)SAYAKA_OK;
  });
}
int sayaka_mac_get_coef_compact(sayaka_mac *h, int32_t which, int32_t dir, double *out) {
  return guarded(h, [&] {
    if (!out || which < 0 || which > 2 || (which < 2 && (dir < 0 || dir >= h->gpu->ndim())))
      return (int)SAYAKA_BAD_INPUT;
    h->gpu->get_coef(which, dir, out);
    return (int)SAYAKA_OK;
  });
}

}  // extern "C"
