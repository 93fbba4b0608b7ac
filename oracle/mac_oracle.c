/*
 * ORACLE -- test infrastructure only, never part of the product path.
 *
 * Plain-C restatement of the SayakaAmr MAC solver hot path (FP64, serial),
 * used by the tests, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline as the checker and the CPU reference timing.  It keeps the
 * reference's data flow -- ghost-cell layers filled level by level, stencils
 * on grown blocks, coarse/fine flux registers (fine-side save, RESTRICT_SUM /
 * AVERAGE to the parent, copy to the coarse neighbour) -- so that it checks
 * the GPU kernels' direct-gather formulation independently.
 *
 * Parity of this restatement is pinned against the reference library itself
 * (golden fixtures written by oracle/ref_dump.cpp; tests/test_oracle.py).
 * Built with -ffp-contract=off so the arithmetic rounds like the reference.
 *
 * Files restated (haloless/SayakaAmr):
 *   src/SayakaTower.cpp:28-187      towers, face registers       orc_build_towers
 *   src/SayakaFillPatch.cpp:34-299  same-level / coarse ghost fill fill_level
 *   src/SayakaMacOperator.cpp:84-137, 1115-1459  operator        orc_apply
 *   src/SayakaMacOperator.cpp:1028-1112, 1191-1323 RB-GS         orc_smooth
 *   src/SayakaTower.cpp:298-415, src/SayakaInterpPatch.cpp:627-691 c/f sync
 *   src/SayakaMacIB.cpp:157-283     weighted restrict / prolong  orc_restrict/prolong
 *   src/SayakaMacOperator.cpp:161-239, 929-1025  face flux       orc_flux
 *   src/SayakaMacOperator.cpp:1470-1594  BC lift                 orc_fix_bc
 *   src/SayakaMacUtil.cpp:9-207     residual, norms, dots, axpby
 *   src/SayakaMacSolver.cpp:164-374, 683-949  bottom, V-cycle, BiCGSTAB
 *   src/SayakaMacCoef.cpp:36-76, src/SayakaMacIB.cpp:34-154  coefficient setup
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PHYS_BNDRY (-20)
enum { FF = 0, BC = 1, FC = 2, CF = 3 };
enum { NEUMANN = 0, DIRICHLET = 1, SIMPLE_FILL = 2 };

typedef struct orc_problem {
  int ndim, nb, nblocks, max_level;
  const int32_t *level, *neighbor, *child, *parent, *which_child, *node_type;
  const double *block_len;
  const int32_t *bc_type; /* [nblocks*6] math BC of physical faces */
  const double *vf;       /* [nblocks*ncell] */
  const double *af[3];    /* [nblocks*nfb] */
  const double *bcoef[3];
  double alpha, beta;
} orc_problem;

typedef struct orc_params {
  int max_iter;
  double tol_rel, tol_abs;
  int n_post;
  int use_precond;
  double bot_tol_rel, bot_tol_abs;
  int bot_max_iter;
  /* relaxation weight of the V-cycle's red-black updates of fluid cells,
   * u_old + omega (u_gs - u_old): 1 is the reference's Gauss-Seidel; other
   * values restate the product's over-relaxed smoother (params.relax_omega) */
  double omega;
} orc_params;

typedef struct orc_info {
  int status, iterations;
  double rnorm0, rnorm;
} orc_info;

/* ------------------------------------------------------------------ */
typedef struct {
  int n;
  int *blocks;
  int *begin, *end; /* [L+1] */
  int *ftype;       /* [n*6] */
} tower_t;

typedef struct {
  const orc_problem *P;
  int nd, nb, G, ncell, gcell, nfb, nblk, finest;
  tower_t *tw; /* [max_level+1] */
  int **lev;   /* tree level lists */
  int *nlev;
  double *dx, *ds, *dv; /* per block metrics */
  double omega;         /* smoother relaxation weight (orc_params.omega) */
} ctx_t;

static int ipow(int a, int e) {
  int r = 1;
  while (e--) r *= a;
  return r;
}

static int gidx(const ctx_t *c, int i, int j, int k) {
  return (i + 1) + c->G * ((j + 1) + c->G * (c->nd == 3 ? k + 1 : 0));
}
static int vidx(const ctx_t *c, int i, int j, int k) { return i + c->nb * (j + c->nb * k); }
static int fidx(const ctx_t *c, int d, int i, int j, int k) {
  const int e0 = c->nb + (d == 0), e1 = c->nb + (d == 1);
  return i + e0 * (j + e1 * k);
}

static void ctx_init(ctx_t *c, const orc_problem *P) {
  c->P = P;
  c->omega = 1.0;
  c->nd = P->ndim;
  c->nb = P->nb;
  c->G = P->nb + 2;
  c->ncell = ipow(P->nb, P->ndim);
  c->gcell = ipow(P->nb + 2, P->ndim);
  c->nfb = (P->nb + 1) * ipow(P->nb, P->ndim - 1);
  c->nblk = P->nblocks;
  c->finest = 0;
  for (int b = 0; b < P->nblocks; b++)
    if (P->level[b] > c->finest) c->finest = P->level[b];
  c->dx = (double *)calloc((size_t)P->nblocks * 3, sizeof(double));
  c->ds = (double *)calloc((size_t)P->nblocks * 3, sizeof(double));
  c->dv = (double *)calloc((size_t)P->nblocks, sizeof(double));
  /* src/SayakaTree.h:277-301 */
  for (int b = 0; b < P->nblocks; b++) {
    double v = 1.0;
    for (int d = 0; d < 3; d++) c->dx[b * 3 + d] = P->block_len[b * 3 + d];
    for (int d = 0; d < c->nd; d++) c->dx[b * 3 + d] /= c->nb;
    for (int d = 0; d < c->nd; d++) v *= c->dx[b * 3 + d];
    for (int d = 0; d < 3; d++) c->ds[b * 3 + d] = 1.0;
    for (int d = 0; d < c->nd; d++) c->ds[b * 3 + d] = v / c->dx[b * 3 + d];
    c->dv[b] = v;
  }
  /* tree level lists, id order (src/SayakaRegrid.cpp:962-976) */
  c->lev = (int **)calloc(P->max_level + 2, sizeof(int *));
  c->nlev = (int *)calloc(P->max_level + 2, sizeof(int));
  for (int l = 1; l <= P->max_level; l++) {
    c->lev[l] = (int *)malloc(sizeof(int) * (P->nblocks + 1));
    for (int b = 0; b < P->nblocks; b++)
      if (P->level[b] == l) c->lev[l][c->nlev[l]++] = b;
  }
  /* towers (src/SayakaTower.cpp:28-187) */
  c->tw = (tower_t *)calloc(P->max_level + 2, sizeof(tower_t));
  for (int L = 1; L <= P->max_level; L++) {
    tower_t *t = &c->tw[L];
    t->blocks = (int *)malloc(sizeof(int) * (P->nblocks + 1));
    t->ftype = (int *)malloc(sizeof(int) * 6 * (P->nblocks + 1));
    t->begin = (int *)calloc(L + 1, sizeof(int));
    t->end = (int *)calloc(L + 1, sizeof(int));
    t->n = 0;
    if (c->nlev[L] == 0) continue;
    for (int l = L; l >= 1; l--) {
      t->begin[l] = t->n;
      for (int q = 0; q < c->nlev[l]; q++) {
        const int b = c->lev[l][q];
        const int leaf = P->node_type[b] == 1;
        if (!(leaf || l == L)) continue;
        for (int f = 0; f < 6; f++) {
          int ty = FF;
          if (f < 2 * c->nd) {
            const int nbr = P->neighbor[b * 6 + f];
            if (nbr <= PHYS_BNDRY)
              ty = BC;
            else if (nbr < 0)
              ty = FC;
            else if (l < L && P->node_type[nbr] != 1)
              ty = CF;
            else
              ty = FF;
          }
          t->ftype[t->n * 6 + f] = ty;
        }
        t->blocks[t->n++] = b;
      }
      t->end[l] = t->n;
    }
  }
}

static void ctx_free(ctx_t *c) {
  for (int L = 1; L <= c->P->max_level; L++) {
    free(c->tw[L].blocks);
    free(c->tw[L].ftype);
    free(c->tw[L].begin);
    free(c->tw[L].end);
    free(c->lev[L]);
  }
  free(c->tw);
  free(c->lev);
  free(c->nlev);
  free(c->dx);
  free(c->ds);
  free(c->dv);
}

/* grown-layout field helpers */
static double *gnew(const ctx_t *c) { return (double *)calloc((size_t)c->nblk * c->gcell, sizeof(double)); }
static double *fnew(const ctx_t *c) { return (double *)calloc((size_t)c->nblk * c->nfb, sizeof(double)); }
static void to_grown(const ctx_t *c, const double *v, double *g) {
  for (int b = 0; b < c->nblk; b++)
    for (int k = 0; k < (c->nd == 3 ? c->nb : 1); k++)
      for (int j = 0; j < c->nb; j++)
        for (int i = 0; i < c->nb; i++)
          g[(size_t)b * c->gcell + gidx(c, i, j, k)] = v[(size_t)b * c->ncell + vidx(c, i, j, k)];
}
static void from_grown(const ctx_t *c, const double *g, double *v) {
  for (int b = 0; b < c->nblk; b++)
    for (int k = 0; k < (c->nd == 3 ? c->nb : 1); k++)
      for (int j = 0; j < c->nb; j++)
        for (int i = 0; i < c->nb; i++)
          v[(size_t)b * c->ncell + vidx(c, i, j, k)] = g[(size_t)b * c->gcell + gidx(c, i, j, k)];
}
#define G_(c, f, b, i, j, k) (f)[(size_t)(b) * (c)->gcell + gidx((c), (i), (j), (k))]
#define V_(c, f, b, i, j, k) (f)[(size_t)(b) * (c)->ncell + vidx((c), (i), (j), (k))]
#define F_(c, f, b, d, i, j, k) (f)[(size_t)(b) * (c)->nfb + fidx((c), (d), (i), (j), (k))]

static int fine_to_crse(int i, int off) { return (i + 64) / 2 - 32 + off; } /* IndexMapping::FineToCrse */

/* ghost fill of every block of a tree level (src/SayakaFillPatch.cpp:34-299):
 * same-level face slabs copied from the neighbour; coarse faces injected
 * from the parent's grown data.  Corners and physical BCs are not filled. */
static void fill_level(const ctx_t *c, int l, double *phi, int only_same) {
  const orc_problem *P = c->P;
  const int nb = c->nb, nd = c->nd;
  for (int q = 0; q < c->nlev[l]; q++) {
    const int b = c->lev[l][q];
    for (int f = 0; f < 2 * nd; f++) {
      const int nbr = P->neighbor[b * 6 + f];
      if (nbr < 0) continue;
      const int d = f >> 1, s = f & 1;
      int lo[3] = {0, 0, 0}, hi[3] = {nb - 1, nd >= 2 ? nb - 1 : 0, nd == 3 ? nb - 1 : 0};
      lo[d] = hi[d] = s ? nb : -1;
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) {
            int src[3] = {i, j, k};
            src[d] = s ? 0 : nb - 1;
            G_(c, phi, b, i, j, k) = G_(c, phi, nbr, src[0], src[1], src[2]);
          }
    }
    if (only_same) continue;
    int has_crse = 0;
    for (int f = 0; f < 2 * nd; f++) {
      const int nbr = P->neighbor[b * 6 + f];
      if (nbr < 0 && nbr > PHYS_BNDRY) has_crse = 1;
    }
    if (!has_crse) continue;
    const int p = P->parent[b], wc = P->which_child[b];
    int off[3] = {0, 0, 0};
    for (int d = 0; d < nd; d++) off[d] = ((wc >> d) & 1) * (nb / 2);
    for (int f = 0; f < 2 * nd; f++) {
      const int nbr = P->neighbor[b * 6 + f];
      if (!(nbr < 0 && nbr > PHYS_BNDRY)) continue;
      const int d = f >> 1, s = f & 1;
      int lo[3] = {0, 0, 0}, hi[3] = {nb - 1, nd >= 2 ? nb - 1 : 0, nd == 3 ? nb - 1 : 0};
      lo[d] = hi[d] = s ? nb : -1;
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) {
            const int ic = fine_to_crse(i, off[0]);
            const int jc = nd >= 2 ? fine_to_crse(j, off[1]) : j;
            const int kc = nd == 3 ? fine_to_crse(k, off[2]) : k;
            G_(c, phi, b, i, j, k) = G_(c, phi, p, ic, jc, kc);
          }
    }
  }
}

/* mg_fillbndry_level (src/SayakaMacUtil.cpp:210-251) */
static void fill_tower(const ctx_t *c, int L, double *phi) {
  const tower_t *t = &c->tw[L];
  for (int l = 1; l <= L; l++) {
    if (l < L && t->end[l + 1] - t->begin[l + 1] <= 0) continue;
    fill_level(c, l, phi, 0);
  }
}

/* syncSubLevelCrseFineFlux (src/SayakaTower.cpp:298-415) */
static void sync_cf(const ctx_t *c, int L, int lf, int dir, double *F, int avg) {
  const orc_problem *P = c->P;
  const tower_t *t = &c->tw[L];
  const int nb = c->nb, nd = c->nd, half = nb / 2;
  if (t->n == 0 || t->end[lf] - t->begin[lf] <= 0 || t->end[lf - 1] - t->begin[lf - 1] <= 0) return;
  const double scale = nd == 3 ? 0.25 : 0.5;
  for (int p = t->begin[lf]; p < t->end[lf]; p++) {
    const int b = t->blocks[p];
    for (int side = 0; side <= 1; side++) {
      if (t->ftype[p * 6 + 2 * dir + side] != FC) continue;
      const int par = P->parent[b], wc = P->which_child[b];
      int off[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
      for (int d = 0; d < nd; d++) {
        off[d] = ((wc >> d) & 1) * half;
        lo[d] = off[d];
        hi[d] = off[d] + half - 1;
      }
      lo[dir] = hi[dir] = side ? off[dir] + half : off[dir];
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) {
            /* restrictFaceBlockData_Average (src/SayakaInterpPatch.cpp:627-691) */
            const int ii1 = dir == 0 ? 0 : 1, jj1 = (dir == 1 || nd < 2) ? 0 : 1, kk1 = (dir == 2 || nd < 3) ? 0 : 1;
            double val = 0;
            for (int kind = -kk1; kind <= kk1; kind += 2)
              for (int jind = -jj1; jind <= jj1; jind += 2)
                for (int iind = -ii1; iind <= ii1; iind += 2) {
                  const int fi = (i - off[0]) * 2 + (dir == 0 ? 0 : (iind + 1) / 2);
                  const int fj = nd >= 2 ? (j - off[1]) * 2 + (dir == 1 ? 0 : (jind + 1) / 2) : j;
                  const int fk = nd == 3 ? (k - off[2]) * 2 + (dir == 2 ? 0 : (kind + 1) / 2) : k;
                  val += F_(c, F, b, dir, fi, fj, fk);
                }
            F_(c, F, par, dir, i, j, k) = avg ? val * scale : val;
          }
    }
  }
  for (int p = t->begin[lf - 1]; p < t->end[lf - 1]; p++) {
    const int b = t->blocks[p];
    for (int side = 0; side <= 1; side++) {
      if (t->ftype[p * 6 + 2 * dir + side] != CF) continue;
      const int nbr = P->neighbor[b * 6 + 2 * dir + side];
      int hi[3] = {nb - 1, nd >= 2 ? nb - 1 : 0, nd == 3 ? nb - 1 : 0};
      hi[dir] = 0;
      for (int k = 0; k <= hi[2]; k++)
        for (int j = 0; j <= hi[1]; j++)
          for (int i = 0; i <= hi[0]; i++) {
            int di[3] = {i, j, k}, si[3] = {i, j, k};
            di[dir] = side ? nb : 0;
            si[dir] = side ? 0 : nb;
            F_(c, F, b, dir, di[0], di[1], di[2]) = F_(c, F, nbr, dir, si[0], si[1], si[2]);
          }
    }
  }
}

static const int IOFF[6] = {-1, 1, 0, 0, 0, 0}, JOFF[6] = {0, 0, -1, 1, 0, 0}, KOFF[6] = {0, 0, 0, 0, -1, 1};

/* cell_eval_coef + B/area corrections (src/SayakaMacOperator.cpp:1115-1167, 1256-1266) */
static void eval_coef(const ctx_t *c, int b, const int *ft, int i, int j, int k, double *off, int *bcf, int *fcf,
                      int *cff) {
  const orc_problem *P = c->P;
  const int ijk[3] = {i, j, k};
  const int range[6] = {0, c->nb - 1, 0, c->nb - 1, 0, c->nb - 1};
  for (int f = 0; f < 2 * c->nd; f++) {
    const int d = f >> 1;
    const double beta = P->beta, ds = c->ds[b * 3 + d], dx = c->dx[b * 3 + d];
    bcf[f] = fcf[f] = cff[f] = 0;
    if (ijk[d] == range[f]) {
      const int ty = ft[f];
      if (ty == FF) {
        off[f] = beta * ds / dx;
      } else if (ty == BC) {
        if (P->bc_type[b * 6 + f] == NEUMANN) {
          off[f] = 0.0;
          bcf[f] = 1;
        } else {
          off[f] = beta * ds / dx;
          bcf[f] = 2;
        }
      } else if (ty == FC) {
        off[f] = beta * ds / (dx * 1.5);
        fcf[f] = 1;
      } else {
        off[f] = beta * ds / (dx * 0.75);
        cff[f] = 1;
      }
    } else {
      off[f] = beta * ds / dx;
    }
  }
  for (int f = 0; f < 2 * c->nd; f++) {
    const int d = f >> 1;
    int fi[3] = {i, j, k};
    fi[d] += f & 1;
    off[f] *= F_(c, P->bcoef[d], b, d, fi[0], fi[1], fi[2]);
    off[f] *= F_(c, P->af[d], b, d, fi[0], fi[1], fi[2]);
  }
}

/* mg_apply_block_usefill (src/SayakaMacOperator.cpp:1325-1459) */
static void apply_block(const ctx_t *c, int b, const int *ft, const double *phi, double *out, double **save) {
  const orc_problem *P = c->P;
  const int nb = c->nb, nd = c->nd;
  for (int k = 0; k < (nd == 3 ? nb : 1); k++)
    for (int j = 0; j < nb; j++)
      for (int i = 0; i < nb; i++) {
        double off[6] = {0}, diag = P->alpha * c->dv[b], offdiag = 0;
        int bcf[6], fcf[6], cff[6];
        eval_coef(c, b, ft, i, j, k, off, bcf, fcf, cff);
        const double phic = G_(c, phi, b, i, j, k);
        for (int f = 0; f < 2 * nd; f++) {
          const int d = f >> 1;
          double val = 0;
          if (!cff[f]) {
            if (bcf[f] == 1) {
              val = 0;
              off[f] = 0;
            } else if (bcf[f] == 2) {
              val = -off[f] * phic;
            } else {
              val = off[f] * G_(c, phi, b, i + IOFF[f], j + JOFF[f], k + KOFF[f]);
            }
          } else {
            int fi[3] = {i, j, k};
            fi[d] += f & 1;
            val = F_(c, save[d], b, d, fi[0], fi[1], fi[2]);
          }
          diag += off[f];
          offdiag += val;
        }
        const double lphi = (phic * diag - offdiag) / c->dv[b];
        const double vf = V_(c, P->vf, b, i, j, k);
        G_(c, out, b, i, j, k) = vf > 0 ? lphi / vf : 0.0;
        for (int f = 0; f < 2 * nd; f++) {
          if (!fcf[f]) continue;
          const int d = f >> 1;
          int fi[3] = {i, j, k};
          fi[d] += f & 1;
          F_(c, save[d], b, d, fi[0], fi[1], fi[2]) = off[f] * phic;
        }
      }
}

/* mg_smooth_block_rbcycle_usefill (src/SayakaMacOperator.cpp:1191-1323) */
static void smooth_block(const ctx_t *c, int b, const int *ft, double *phi, const double *rhs, double **save,
                         int rb) {
  const orc_problem *P = c->P;
  const int nb = c->nb, nd = c->nd;
  for (int k = 0; k < (nd == 3 ? nb : 1); k++)
    for (int j = 0; j < nb; j++)
      for (int i = 0; i < nb; i++) {
        if ((i + j + k) % 2 != rb) continue;
        double off[6] = {0}, diag = P->alpha * c->dv[b], offdiag = 0;
        int bcf[6], fcf[6], cff[6];
        eval_coef(c, b, ft, i, j, k, off, bcf, fcf, cff);
        for (int f = 0; f < 2 * nd; f++) {
          const int d = f >> 1;
          double val = 0;
          if (!cff[f]) {
            if (bcf[f] == 1) {
              val = 0;
              off[f] = 0;
            } else if (bcf[f] == 2) {
              val = 0;
              off[f] *= 2.0;
            } else {
              val = off[f] * G_(c, phi, b, i + IOFF[f], j + JOFF[f], k + KOFF[f]);
            }
          } else {
            int fi[3] = {i, j, k};
            fi[d] += f & 1;
            val = F_(c, save[d], b, d, fi[0], fi[1], fi[2]);
          }
          diag += off[f];
          offdiag += val;
        }
        const double r = G_(c, rhs, b, i, j, k), vf = V_(c, P->vf, b, i, j, k);
        double unew = 0;
        if (vf > 0) unew = (r * c->dv[b] * vf + offdiag) / diag;
        if (vf > 0 && c->omega != 1.0) unew = c->omega * unew + (1.0 - c->omega) * G_(c, phi, b, i, j, k);
        G_(c, phi, b, i, j, k) = unew;
        for (int f = 0; f < 2 * nd; f++) {
          if (!fcf[f]) continue;
          const int d = f >> 1;
          int fi[3] = {i, j, k};
          fi[d] += f & 1;
          F_(c, save[d], b, d, fi[0], fi[1], fi[2]) = off[f] * unew;
        }
      }
}

typedef struct {
  double *save[3];
} regs_t;
static void regs_new(const ctx_t *c, regs_t *r) {
  for (int d = 0; d < 3; d++) r->save[d] = d < c->nd ? fnew(c) : NULL;
}
static void regs_free(regs_t *r) {
  for (int d = 0; d < 3; d++) free(r->save[d]);
}

/* mg_apply_level (src/SayakaMacOperator.cpp:84-137) on grown fields */
static void g_apply(const ctx_t *c, int L, double *in, double *out, regs_t *R) {
  const tower_t *t = &c->tw[L];
  if (c->nlev[L] == 0) return;
  fill_tower(c, L, in);
  for (int l = L; l >= 1; l--) {
    for (int p = t->begin[l]; p < t->end[l]; p++) apply_block(c, t->blocks[p], &t->ftype[p * 6], in, out, R->save);
    if (l > 1)
      for (int d = 0; d < c->nd; d++) sync_cf(c, L, l, d, R->save[d], 0);
  }
}

/* mg_residual_level (src/SayakaMacUtil.cpp:9-49) */
static void g_residual(const ctx_t *c, int L, double *res, double *phi, const double *rhs, regs_t *R) {
  const tower_t *t = &c->tw[L];
  g_apply(c, L, phi, res, R);
  for (int p = 0; p < t->n; p++) {
    const int b = t->blocks[p];
    for (int k = 0; k < (c->nd == 3 ? c->nb : 1); k++)
      for (int j = 0; j < c->nb; j++)
        for (int i = 0; i < c->nb; i++) {
          const double lphi = G_(c, res, b, i, j, k);
          G_(c, res, b, i, j, k) = V_(c, c->P->vf, b, i, j, k) > 0 ? G_(c, rhs, b, i, j, k) - lphi : 0.0;
        }
  }
}

/* mg_smooth_level_usefill (src/SayakaMacOperator.cpp:1028-1112) */
static void g_smooth(const ctx_t *c, int L, double *phi, const double *rhs, regs_t *R) {
  const tower_t *t = &c->tw[L];
  if (c->nlev[L] == 0) return;
  fill_tower(c, L, phi);
  for (int d = 0; d < c->nd; d++) memset(R->save[d], 0, sizeof(double) * (size_t)c->nblk * c->nfb);
  for (int l = L; l >= 1; l--) {
    if (t->begin[l] >= t->end[l]) break;
    for (int rb = 0; rb < 2; rb++) {
      fill_level(c, l, phi, 1);
      for (int p = t->begin[l]; p < t->end[l]; p++)
        smooth_block(c, t->blocks[p], &t->ftype[p * 6], phi, rhs, R->save, rb);
    }
    if (l > 1)
      for (int d = 0; d < c->nd; d++) sync_cf(c, L, l, d, R->save[d], 0);
  }
}

/* mg_restict_wgt (src/SayakaMacIB.cpp:157-232) */
static void g_restrict(const ctx_t *c, int lc, double *phi, double *tmp) {
  const orc_problem *P = c->P;
  if (lc >= P->max_level || c->nlev[lc] == 0 || c->nlev[lc + 1] == 0) return;
  const int nb = c->nb, nd = c->nd, half = nb / 2, lf = lc + 1;
  for (int q = 0; q < c->nlev[lf]; q++) {
    const int b = c->lev[lf][q];
    memcpy(&tmp[(size_t)b * c->gcell], &phi[(size_t)b * c->gcell], sizeof(double) * c->gcell);
    for (int k = 0; k < (nd == 3 ? nb : 1); k++)
      for (int j = 0; j < nb; j++)
        for (int i = 0; i < nb; i++) G_(c, phi, b, i, j, k) *= V_(c, P->vf, b, i, j, k);
  }
  const double wgt = 1.0 / (1 << nd);
  for (int q = 0; q < c->nlev[lc]; q++) {
    const int b = c->lev[lc][q];
    if (P->node_type[b] == 1) continue;
    for (int ch = 0; ch < (1 << nd); ch++) {
      const int cb = P->child[b * 8 + ch];
      int off[3] = {0, 0, 0};
      for (int d = 0; d < nd; d++) off[d] = ((ch >> d) & 1) * half;
      for (int kc = off[2]; kc < off[2] + (nd == 3 ? half : 1); kc++)
        for (int jc = off[1]; jc < off[1] + half; jc++)
          for (int ic = off[0]; ic < off[0] + half; ic++) {
            double sum = 0;
            for (int kk = 0; kk <= (nd == 3 ? 1 : 0); kk++)
              for (int jj = 0; jj <= 1; jj++)
                for (int ii = 0; ii <= 1; ii++)
                  sum += G_(c, phi, cb, (ic - off[0]) * 2 + ii, (jc - off[1]) * 2 + jj,
                            nd == 3 ? (kc - off[2]) * 2 + kk : 0);
            G_(c, phi, b, ic, jc, kc) = sum * wgt;
          }
    }
    for (int k = 0; k < (nd == 3 ? nb : 1); k++)
      for (int j = 0; j < nb; j++)
        for (int i = 0; i < nb; i++) {
          const double vf = V_(c, P->vf, b, i, j, k);
          if (vf > 0)
            G_(c, phi, b, i, j, k) /= vf;
          else
            G_(c, phi, b, i, j, k) = 0;
        }
  }
  for (int q = 0; q < c->nlev[lf]; q++) {
    const int b = c->lev[lf][q];
    for (int k = 0; k < (nd == 3 ? nb : 1); k++)
      for (int j = 0; j < nb; j++)
        for (int i = 0; i < nb; i++) G_(c, phi, b, i, j, k) = G_(c, tmp, b, i, j, k);
  }
}

/* mg_prolong_wgt (src/SayakaMacIB.cpp:234-283) */
static void g_prolong(const ctx_t *c, int lf, double *phi) {
  const orc_problem *P = c->P;
  if (lf <= 1 || c->nlev[lf] == 0) return;
  const int nb = c->nb, nd = c->nd;
  for (int q = 0; q < c->nlev[lf]; q++) {
    const int b = c->lev[lf][q], p = P->parent[b], wc = P->which_child[b];
    int off[3] = {0, 0, 0};
    for (int d = 0; d < nd; d++) off[d] = ((wc >> d) & 1) * (nb / 2);
    for (int k = 0; k < (nd == 3 ? nb : 1); k++)
      for (int j = 0; j < nb; j++)
        for (int i = 0; i < nb; i++) {
          const double v = G_(c, phi, p, fine_to_crse(i, off[0]), fine_to_crse(j, off[1]),
                              nd == 3 ? fine_to_crse(k, off[2]) : 0);
          G_(c, phi, b, i, j, k) = V_(c, P->vf, b, i, j, k) > 0 ? v : 0.0;
        }
  }
}

/* ---- tower vector ops in the reference's order (src/SayakaMacUtil.cpp) ---- */
static double t_norm(const ctx_t *c, int L, const double *x) {
  const tower_t *t = &c->tw[L];
  double m = 0;
  for (int p = 0; p < t->n; p++) {
    const int b = t->blocks[p];
    double r = fabs(G_(c, x, b, 0, 0, 0));
    for (int k = 0; k < (c->nd == 3 ? c->nb : 1); k++)
      for (int j = 0; j < c->nb; j++)
        for (int i = 0; i < c->nb; i++) {
          const double v = fabs(G_(c, x, b, i, j, k));
          if (v > r) r = v;
        }
    if (r > m) m = r;
  }
  return m;
}
static double t_dot(const ctx_t *c, int L, const double *a, const double *bb) {
  const tower_t *t = &c->tw[L];
  double s = 0;
  for (int p = 0; p < t->n; p++) {
    const int b = t->blocks[p];
    double sb = 0;
    for (int k = 0; k < (c->nd == 3 ? c->nb : 1); k++)
      for (int j = 0; j < c->nb; j++)
        for (int i = 0; i < c->nb; i++) sb += G_(c, a, b, i, j, k) * G_(c, bb, b, i, j, k);
    s += sb;
  }
  return s;
}
static void t_axpby(const ctx_t *c, int L, double *out, double a, const double *x, double bcoef, const double *y) {
  const tower_t *t = &c->tw[L];
  for (int p = 0; p < t->n; p++) {
    const int b = t->blocks[p];
    for (int k = 0; k < (c->nd == 3 ? c->nb : 1); k++)
      for (int j = 0; j < c->nb; j++)
        for (int i = 0; i < c->nb; i++) G_(c, out, b, i, j, k) = a * G_(c, x, b, i, j, k) + bcoef * G_(c, y, b, i, j, k);
  }
}
static void t_copy(const ctx_t *c, int L, double *dst, const double *src) {
  const tower_t *t = &c->tw[L];
  for (int p = 0; p < t->n; p++) {
    const int b = t->blocks[p];
    for (int k = 0; k < (c->nd == 3 ? c->nb : 1); k++)
      for (int j = 0; j < c->nb; j++)
        for (int i = 0; i < c->nb; i++) G_(c, dst, b, i, j, k) = G_(c, src, b, i, j, k);
  }
}
static void t_zero(const ctx_t *c, int L, double *dst) {
  const tower_t *t = &c->tw[L];
  for (int p = 0; p < t->n; p++) memset(&dst[(size_t)t->blocks[p] * c->gcell], 0, sizeof(double) * c->gcell);
}

/* ---- solver state ---- */
enum { B_RHS, B_SOL, B_RESID, B_CORR, B_TMP, X0, X, R, RHAT, P_, PHAT, S_, SHAT, V_v, T_v,
       BX0, BX, BR, BRHAT, BP, BS, BV, BT, NVEC };
typedef struct {
  ctx_t c;
  regs_t R;
  double *v[NVEC];
  orc_params prm;
} solver_t;

static void solver_init(solver_t *s, const orc_problem *P, const orc_params *prm) {
  ctx_init(&s->c, P);
  regs_new(&s->c, &s->R);
  for (int i = 0; i < NVEC; i++) s->v[i] = gnew(&s->c);
  if (prm) {
    s->prm = *prm;
    if (prm->omega > 0.0) s->c.omega = prm->omega;
  }
}
static void solver_free(solver_t *s) {
  for (int i = 0; i < NVEC; i++) free(s->v[i]);
  regs_free(&s->R);
  ctx_free(&s->c);
}

static int bicgstab(solver_t *s, int L, double *sol, double *rhs, double tol_rel, double tol_abs, int max_iter,
                    int precond, int bottom, orc_info *info);

/* mg_solve_bottom (src/SayakaMacSolver.cpp:164-242); the bottom keeps its
 * own BiCGSTAB vectors (the reference shares them with the outer solve,
 * which is only safe -- and only used here -- without level-1 leaves) */
static int bottom_solve(solver_t *s) {
  orc_info bi;
  t_zero(&s->c, 1, s->v[B_CORR]);
  return bicgstab(s, 1, s->v[B_CORR], s->v[B_RESID], s->prm.bot_tol_rel, s->prm.bot_tol_abs, s->prm.bot_max_iter, 0,
                  1, &bi);
}

/* mg_precond_level -> mg_relax_vcycle, fixed_iter = 1
 * (src/SayakaMacSolver.cpp:924-949, 245-374) */
static void precond(solver_t *s, int L, double *sol, double *rhs) {
  ctx_t *c = &s->c;
  t_zero(c, L, sol);
  t_copy(c, L, s->v[B_SOL], sol);
  g_residual(c, L, s->v[B_RESID], s->v[B_SOL], rhs, &s->R);
  t_zero(c, L, s->v[B_CORR]);
  for (int l = L; l >= 2; l--) g_restrict(c, l - 1, s->v[B_RESID], s->v[B_TMP]);
  if (bottom_solve(s) != 0) {
    t_copy(c, L, sol, s->v[B_SOL]);
    return;
  }
  for (int l = 2; l <= L; l++) {
    g_prolong(c, l, s->v[B_CORR]);
    for (int k = 0; k < s->prm.n_post; k++) g_smooth(c, l, s->v[B_CORR], s->v[B_RESID], &s->R);
  }
  t_axpby(c, L, s->v[B_SOL], 1.0, s->v[B_SOL], 1.0, s->v[B_CORR]);
  t_copy(c, L, sol, s->v[B_SOL]);
}

/* cg_solve_level (src/SayakaMacSolver.cpp:683-920) */
static int bicgstab(solver_t *s, int L, double *sol, double *rhs, double tol_rel, double tol_abs, int max_iter,
                    int use_pc, int bottom, orc_info *info) {
  ctx_t *c = &s->c;
  double *x0 = s->v[bottom ? BX0 : X0], *x = s->v[bottom ? BX : X], *r = s->v[bottom ? BR : R];
  double *rhat = s->v[bottom ? BRHAT : RHAT], *p = s->v[bottom ? BP : P_], *sv = s->v[bottom ? BS : S_];
  double *v = s->v[bottom ? BV : V_v], *tt = s->v[bottom ? BT : T_v];
  double *phat = bottom ? p : s->v[PHAT], *shat = bottom ? sv : s->v[SHAT];
  if (L == 1) use_pc = 0;
  t_copy(c, L, x0, sol);
  g_residual(c, L, r, x0, rhs, &s->R);
  t_copy(c, L, rhat, r);
  t_zero(c, L, x);
  const double rnorm0 = t_norm(c, L, r);
  info->rnorm0 = info->rnorm = rnorm0;
  info->iterations = 0;
  info->status = 0;
  if (rnorm0 == 0) return 0;
  double rho1 = 0, alpha = 0, omega = 0;
  int conv = 0, stat = 0, iter;
  for (iter = 1; iter <= max_iter; iter++) {
    const double rho = t_dot(c, L, rhat, r);
    if (rho == 0) {
      stat = 1;
      break;
    }
    if (iter == 1) {
      t_copy(c, L, p, r);
    } else {
      const double beta = (rho / rho1) * (alpha / omega);
      t_axpby(c, L, p, 1.0, p, -omega, v);
      t_axpby(c, L, p, 1.0, r, beta, p);
    }
    if (use_pc)
      precond(s, L, phat, p);
    else if (phat != p)
      t_copy(c, L, phat, p);
    g_apply(c, L, phat, v, &s->R);
    alpha = t_dot(c, L, rhat, v);
    if (alpha == 0) {
      stat = 1;
      break;
    }
    alpha = rho / alpha;
    t_axpby(c, L, sv, 1.0, r, -alpha, v);
    t_axpby(c, L, x, 1.0, x, alpha, phat);
    double rn = t_norm(c, L, sv);
    info->rnorm = rn;
    if (rn < rnorm0 * tol_rel || rn < tol_abs) {
      conv = 1;
      break;
    }
    if (use_pc)
      precond(s, L, shat, sv);
    else if (shat != sv)
      t_copy(c, L, shat, sv);
    g_apply(c, L, shat, tt, &s->R);
    const double tds = t_dot(c, L, tt, sv), tdt = t_dot(c, L, tt, tt);
    if (tdt == 0) {
      stat = 1;
      break;
    }
    omega = tds / tdt;
    t_axpby(c, L, x, 1.0, x, omega, shat);
    t_axpby(c, L, r, 1.0, sv, -omega, tt);
    rn = t_norm(c, L, r);
    info->rnorm = rn;
    if (rn < rnorm0 * tol_rel + tol_abs) {
      conv = 1;
      break;
    }
    if (omega == 0) {
      stat = 1;
      break;
    }
    rho1 = rho;
  }
  info->iterations = iter > max_iter ? max_iter : iter;
  if (conv) {
    t_axpby(c, L, x0, 1.0, x0, 1.0, x);
    t_copy(c, L, sol, x0);
  }
  info->status = stat ? 1 : (conv ? 0 : 2);
  return stat;
}

/* ================================================================== */
/* exported entry points (compact all-block arrays)                    */

int orc_apply(const orc_problem *P, int L, const double *x, double *y) {
  solver_t s;
  solver_init(&s, P, NULL);
  to_grown(&s.c, x, s.v[P_]);
  g_apply(&s.c, L, s.v[P_], s.v[V_v], &s.R);
  from_grown(&s.c, s.v[V_v], y);
  solver_free(&s);
  return 0;
}

int orc_residual(const orc_problem *P, int L, const double *x, const double *rhs, double *r) {
  solver_t s;
  solver_init(&s, P, NULL);
  to_grown(&s.c, x, s.v[P_]);
  to_grown(&s.c, rhs, s.v[S_]);
  g_residual(&s.c, L, s.v[T_v], s.v[P_], s.v[S_], &s.R);
  from_grown(&s.c, s.v[T_v], r);
  solver_free(&s);
  return 0;
}

int orc_smooth(const orc_problem *P, int L, const double *phi, const double *rhs, double *out) {
  solver_t s;
  solver_init(&s, P, NULL);
  to_grown(&s.c, phi, s.v[B_CORR]);
  to_grown(&s.c, rhs, s.v[B_RESID]);
  g_smooth(&s.c, L, s.v[B_CORR], s.v[B_RESID], &s.R);
  from_grown(&s.c, s.v[B_CORR], out);
  solver_free(&s);
  return 0;
}

/* orc_smooth with relaxed updates of the fluid cells (orc_params.omega) */
int orc_smooth_relaxed(const orc_problem *P, int L, const double *phi, const double *rhs, double omega,
                       double *out) {
  solver_t s;
  solver_init(&s, P, NULL);
  s.c.omega = omega;
  to_grown(&s.c, phi, s.v[B_CORR]);
  to_grown(&s.c, rhs, s.v[B_RESID]);
  g_smooth(&s.c, L, s.v[B_CORR], s.v[B_RESID], &s.R);
  from_grown(&s.c, s.v[B_CORR], out);
  solver_free(&s);
  return 0;
}

int orc_restrict_sweep(const orc_problem *P, const double *in, double *out) {
  solver_t s;
  solver_init(&s, P, NULL);
  to_grown(&s.c, in, s.v[B_RESID]);
  for (int l = s.c.finest; l >= 2; l--) g_restrict(&s.c, l - 1, s.v[B_RESID], s.v[B_TMP]);
  from_grown(&s.c, s.v[B_RESID], out);
  solver_free(&s);
  return 0;
}

int orc_prolong_sweep(const orc_problem *P, const double *in, double *out) {
  solver_t s;
  solver_init(&s, P, NULL);
  to_grown(&s.c, in, s.v[B_CORR]);
  for (int l = 2; l <= s.c.finest; l++) g_prolong(&s.c, l, s.v[B_CORR]);
  from_grown(&s.c, s.v[B_CORR], out);
  solver_free(&s);
  return 0;
}

/* mg_flux_level + mg_flux_block_usefill (src/SayakaMacOperator.cpp:161-239, 929-1025) */
int orc_flux(const orc_problem *P, int dir, const double *phi_in, double *flux) {
  solver_t s;
  solver_init(&s, P, NULL);
  ctx_t *c = &s.c;
  double *phi = s.v[P_];
  to_grown(c, phi_in, phi);
  double *fl = fnew(c);
  const int L = c->finest, nb = c->nb, nd = c->nd;
  const tower_t *t = &c->tw[L];
  fill_tower(c, L, phi);
  for (int l = L; l >= 1; l--) {
    for (int p = t->begin[l]; p < t->end[l]; p++) {
      const int b = t->blocks[p];
      const double dh = c->dx[b * 3 + dir];
      const int ii = dir == 0, jj = dir == 1, kk = dir == 2;
      for (int k = 0; k < (nd == 3 ? nb + kk : 1); k++)
        for (int j = 0; j < nb + jj; j++)
          for (int i = 0; i < nb + ii; i++) {
            const int ijk = dir == 0 ? i : (dir == 1 ? j : k);
            const int side = ijk == 0 ? 0 : (ijk == nb ? 1 : -1);
            const double d = G_(c, phi, b, i, j, k) - G_(c, phi, b, i - ii, j - jj, k - kk);
            if (side >= 0) {
              const int ty = t->ftype[p * 6 + 2 * dir + side];
              if (ty == BC)
                F_(c, fl, b, dir, i, j, k) = 0;
              else if (ty == FF)
                F_(c, fl, b, dir, i, j, k) = -d / dh;
              else if (ty == FC)
                F_(c, fl, b, dir, i, j, k) = -d / (dh * 1.5);
            } else {
              F_(c, fl, b, dir, i, j, k) = -d / dh;
            }
          }
    }
    if (l > 1) sync_cf(c, L, l, dir, fl, 1);
  }
  memcpy(flux, fl, sizeof(double) * (size_t)c->nblk * c->nfb);
  free(fl);
  solver_free(&s);
  return 0;
}

/* fixBC / fixBlockBC (src/SayakaMacOperator.cpp:1470-1594); phi_grown holds
 * [block][grown box] with one ghost layer */
int orc_fix_bc(const orc_problem *P, const double *phi_grown, double *rhs) {
  solver_t s;
  solver_init(&s, P, NULL);
  ctx_t *c = &s.c;
  const int L = c->finest, nb = c->nb, nd = c->nd;
  const tower_t *t = &c->tw[L];
  for (int p = 0; p < t->n; p++) {
    const int b = t->blocks[p];
    for (int f = 0; f < 2 * nd; f++) {
      if (t->ftype[p * 6 + f] != BC) continue;
      const int bct = P->bc_type[b * 6 + f];
      const int d = f >> 1, sd = f & 1;
      int lo[3] = {0, 0, 0}, hi[3] = {nb - 1, nb - 1, nd == 3 ? nb - 1 : 0};
      lo[d] = hi[d] = sd ? nb - 1 : 0;
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
          for (int i = lo[0]; i <= hi[0]; i++) {
            const double phi0 = G_(c, phi_grown, b, i, j, k);
            const double phi1 = G_(c, phi_grown, b, i + IOFF[f], j + JOFF[f], k + KOFF[f]);
            int fi[3] = {i, j, k};
            fi[d] += sd;
            double coef = P->beta * c->ds[b * 3 + d] / c->dx[b * 3 + d];
            coef *= F_(c, P->bcoef[d], b, d, fi[0], fi[1], fi[2]);
            coef *= F_(c, P->af[d], b, d, fi[0], fi[1], fi[2]);
            double corr = 0;
            if (bct == DIRICHLET) {
              const double pbc = 0.5 * (phi0 + phi1);
              corr = pbc * 2.0 * coef;
            } else if (bct == SIMPLE_FILL) {
              corr = phi1 * 2.0 * coef;
            }
            const double vf = V_(c, P->vf, b, i, j, k);
            if (vf > 0) {
              corr /= (c->dv[b] * vf);
              V_(c, rhs, b, i, j, k) += corr;
            }
          }
    }
  }
  solver_free(&s);
  return 0;
}

int orc_vcycle(const orc_problem *P, const orc_params *prm, const double *p_in, double *phat) {
  solver_t s;
  solver_init(&s, P, prm);
  to_grown(&s.c, p_in, s.v[P_]);
  precond(&s, s.c.finest, s.v[PHAT], s.v[P_]);
  from_grown(&s.c, s.v[PHAT], phat);
  solver_free(&s);
  return 0;
}

/* cg_solve (src/SayakaMacSolver.cpp:455-680): sol holds the initial guess */
int orc_cg_solve(const orc_problem *P, const orc_params *prm, const double *rhs, double *sol, orc_info *info) {
  solver_t s;
  solver_init(&s, P, prm);
  to_grown(&s.c, rhs, s.v[B_RHS]);
  to_grown(&s.c, sol, s.v[B_SOL]);
  const int st = bicgstab(&s, s.c.finest, s.v[B_SOL], s.v[B_RHS], prm->tol_rel, prm->tol_abs, prm->max_iter,
                          prm->use_precond, 0, info);
  from_grown(&s.c, s.v[B_SOL], sol);
  solver_free(&s);
  return st;
}

/* mg_solve (src/SayakaMacSolver.cpp:43-162): stand-alone V-cycles on the
 * finest tower.  RESID = RHS - L(SOL); every iteration clears CORR, restricts
 * RESID down to level 1, solves the bottom, prolongs and post-smooths up,
 * adds CORR to SOL and recomputes RESID and its L-inf norm; stops when
 * |r| < |r0| tol_rel + tol_abs or after max_iter iterations.  sol holds the
 * initial guess.  Returns 1 when the bottom solve breaks down (the reference
 * exits), else 0; info->status 2 when it did not converge. */
int orc_mg_solve(const orc_problem *P, const orc_params *prm, const double *rhs, double *sol, orc_info *info) {
  solver_t s;
  solver_init(&s, P, prm);
  ctx_t *c = &s.c;
  const int L = c->finest;
  to_grown(c, rhs, s.v[B_RHS]);
  to_grown(c, sol, s.v[B_SOL]);
  g_residual(c, L, s.v[B_RESID], s.v[B_SOL], s.v[B_RHS], &s.R);
  const double r0 = t_norm(c, L, s.v[B_RESID]);
  double rn = r0;
  int it = 0, conv = 0, st = 0;
  for (it = 1; it <= prm->max_iter; it++) {
    memset(s.v[B_CORR], 0, sizeof(double) * (size_t)c->nblk * c->gcell);
    for (int l = L; l >= 2; l--) g_restrict(c, l - 1, s.v[B_RESID], s.v[B_TMP]);
    if (bottom_solve(&s) != 0) {
      st = 1;
      break;
    }
    for (int l = 2; l <= L; l++) {
      g_prolong(c, l, s.v[B_CORR]);
      for (int k = 0; k < prm->n_post; k++) g_smooth(c, l, s.v[B_CORR], s.v[B_RESID], &s.R);
    }
    t_axpby(c, L, s.v[B_SOL], 1.0, s.v[B_SOL], 1.0, s.v[B_CORR]);
    g_residual(c, L, s.v[B_RESID], s.v[B_SOL], s.v[B_RHS], &s.R);
    rn = t_norm(c, L, s.v[B_RESID]);
    if (rn < r0 * prm->tol_rel + prm->tol_abs) {
      conv = 1;
      break;
    }
  }
  if (it > prm->max_iter) it = prm->max_iter;
  from_grown(c, s.v[B_SOL], sol);
  info->status = st ? 1 : (conv ? 0 : 2);
  info->iterations = it;
  info->rnorm0 = r0;
  info->rnorm = rn;
  solver_free(&s);
  return st;
}

/* relax_solve (src/SayakaMacSolver.cpp:377-452): red-black Gauss-Seidel
 * sweeps of the finest tower on SOL with RHS (mg_smooth_level), the residual's
 * L-inf norm after each, until |r| < |r0| tol_rel + tol_abs or max_iter */
int orc_relax_solve(const orc_problem *P, const orc_params *prm, const double *rhs, double *sol, orc_info *info) {
  solver_t s;
  solver_init(&s, P, prm);
  ctx_t *c = &s.c;
  const int L = c->finest;
  to_grown(c, rhs, s.v[B_RHS]);
  to_grown(c, sol, s.v[B_SOL]);
  g_residual(c, L, s.v[B_RESID], s.v[B_SOL], s.v[B_RHS], &s.R);
  const double r0 = t_norm(c, L, s.v[B_RESID]);
  double rn = r0;
  int it = 0, conv = 0;
  for (it = 1; it <= prm->max_iter; it++) {
    g_smooth(c, L, s.v[B_SOL], s.v[B_RHS], &s.R);
    g_residual(c, L, s.v[B_RESID], s.v[B_SOL], s.v[B_RHS], &s.R);
    rn = t_norm(c, L, s.v[B_RESID]);
    if (rn < r0 * prm->tol_rel + prm->tol_abs) {
      conv = 1;
      break;
    }
  }
  if (it > prm->max_iter) it = prm->max_iter;
  from_grown(c, s.v[B_SOL], sol);
  info->status = conv ? 0 : 2;
  info->iterations = it;
  info->rnorm0 = r0;
  info->rnorm = rn;
  solver_free(&s);
  return 0;
}

/* tower block list, begin/end and face types (for table checks) */
int orc_tower(const orc_problem *P, int L, int32_t *blocks, int32_t *n, int32_t *begin_end, int32_t *ftypes) {
  ctx_t c;
  ctx_init(&c, P);
  const tower_t *t = &c.tw[L];
  *n = t->n;
  for (int p = 0; p < t->n; p++) {
    blocks[p] = t->blocks[p];
    for (int f = 0; f < 6; f++) ftypes[p * 6 + f] = t->ftype[p * 6 + f];
  }
  for (int l = 1; l <= L; l++) {
    begin_end[2 * (l - 1)] = t->n ? t->begin[l] : 0;
    begin_end[2 * (l - 1) + 1] = t->n ? t->end[l] : 0;
  }
  ctx_free(&c);
  return 0;
}

/* AVG restriction of face data of direction dir onto the non-leaf blocks of
 * levels finest-1 .. 1 (src/SayakaFillPatch.cpp:401-447 with
 * src/SayakaInterpPatch.cpp:627-691) */
static void restrict_face_levels(const ctx_t *c, int dir, double *F) {
  const orc_problem *P = c->P;
  const int nb = c->nb, nd = c->nd, half = nb / 2;
  const double scale = nd == 3 ? 0.25 : 0.5;
  for (int l = c->finest - 1; l >= 1; l--)
    for (int q = 0; q < c->nlev[l]; q++) {
      const int b = c->lev[l][q];
      if (P->node_type[b] == 1) continue;
      for (int ch = 0; ch < (1 << nd); ch++) {
        const int cb = P->child[b * 8 + ch];
        int off[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        for (int d = 0; d < nd; d++) {
          off[d] = ((ch >> d) & 1) * half;
          lo[d] = off[d];
          hi[d] = off[d] + half - 1;
        }
        hi[dir] += 1;
        for (int k = lo[2]; k <= hi[2]; k++)
          for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) {
              const int ii1 = dir == 0 ? 0 : 1, jj1 = (dir == 1 || nd < 2) ? 0 : 1, kk1 = (dir == 2 || nd < 3) ? 0 : 1;
              double val = 0;
              for (int kind = -kk1; kind <= kk1; kind += 2)
                for (int jind = -jj1; jind <= jj1; jind += 2)
                  for (int iind = -ii1; iind <= ii1; iind += 2) {
                    const int fi = (i - off[0]) * 2 + (dir == 0 ? 0 : (iind + 1) / 2);
                    const int fj = nd >= 2 ? (j - off[1]) * 2 + (dir == 1 ? 0 : (jind + 1) / 2) : j;
                    const int fk = nd == 3 ? (k - off[2]) * 2 + (dir == 2 ? 0 : (kind + 1) / 2) : k;
                    val += F_(c, F, cb, dir, fi, fj, fk);
                  }
              F_(c, F, b, dir, i, j, k) = val * scale;
            }
      }
    }
}

/* AVG restriction of cell data onto non-leaf blocks, finest-1 .. 1 */
static void restrict_cell_levels(const ctx_t *c, double *V) {
  const orc_problem *P = c->P;
  const int nb = c->nb, nd = c->nd, half = nb / 2;
  const double wgt = 1.0 / (1 << nd);
  for (int l = c->finest - 1; l >= 1; l--)
    for (int q = 0; q < c->nlev[l]; q++) {
      const int b = c->lev[l][q];
      if (P->node_type[b] == 1) continue;
      for (int ch = 0; ch < (1 << nd); ch++) {
        const int cb = P->child[b * 8 + ch];
        int off[3] = {0, 0, 0};
        for (int d = 0; d < nd; d++) off[d] = ((ch >> d) & 1) * half;
        for (int kc = off[2]; kc < off[2] + (nd == 3 ? half : 1); kc++)
          for (int jc = off[1]; jc < off[1] + half; jc++)
            for (int ic = off[0]; ic < off[0] + half; ic++) {
              double sum = 0;
              for (int kk = 0; kk <= (nd == 3 ? 1 : 0); kk++)
                for (int jj = 0; jj <= 1; jj++)
                  for (int ii = 0; ii <= 1; ii++)
                    sum += V_(c, V, cb, (ic - off[0]) * 2 + ii, (jc - off[1]) * 2 + jj,
                              nd == 3 ? (kc - off[2]) * 2 + kk : 0);
              V_(c, V, b, ic, jc, kc) = sum * wgt;
            }
      }
    }
}

/* setCoefB (src/SayakaMacCoef.cpp:36-76) and the fraction part of
 * calcIBFracByLS (src/SayakaMacIB.cpp:69-96): the arrays hold leaf values
 * on entry (other blocks are overwritten); c/f AVG sync on the finest tower,
 * then AVG restriction to the parents.  Any pointer may be NULL. */
int orc_setup_coefficients(const orc_problem *P, double *vf, double *af0, double *af1, double *af2, double *b0,
                           double *b1, double *b2) {
  ctx_t c;
  ctx_init(&c, P);
  double *af[3] = {af0, af1, af2}, *bc[3] = {b0, b1, b2};
  for (int d = 0; d < c.nd; d++) {
    if (bc[d]) {
      for (int l = c.finest; l >= 2; l--) sync_cf(&c, c.finest, l, d, bc[d], 1);
      restrict_face_levels(&c, d, bc[d]);
    }
  }
  for (int d = 0; d < c.nd; d++)
    if (af[d])
      for (int l = c.finest; l >= 2; l--) sync_cf(&c, c.finest, l, d, af[d], 1);
  if (vf) restrict_cell_levels(&c, vf);
  for (int d = 0; d < c.nd; d++)
    if (af[d]) restrict_face_levels(&c, d, af[d]);
  ctx_free(&c);
  return 0;
}
