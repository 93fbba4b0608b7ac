// Golden-vector generator: drives the UNMODIFIED reference library
// (haloless/SayakaAmr, compiled by oracle/Makefile into oracle/_ref/) through its
// own public API and dumps tree tables, MG towers, face registers and the
// results of every hot-path routine for seeded synthetic inputs.
//
// This file is test infrastructure (the oracle), never part of the product.
// It is compiled twice (SAYAKA_SPACEDIM=2 and =3) against the reference
// sources where they lie; it only *calls* the reference.
//
// Output format (read by tests/golden_io.py): "SYKG" magic, then records of
//   u32 name_len | name | u8 dtype (0=i32, 1=f64) | u64 count | payload.

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cstdint>
#include <random>
#include <string>
#include <vector>
#include <memory>

#include "SayakaTree.h"
#include "SayakaTreeData.h"
#include "SayakaBoundaryPatch.h"
#include "SayakaFillPatch.h"
#include "SayakaTower.h"
#include "SayakaMacSolver.h"

using namespace sayaka;

// ---------------------------------------------------------------------------
// dump container
struct Dump {
	FILE *fp = nullptr;
	explicit Dump(const char *path) {
		fp = fopen(path, "wb");
		if (!fp) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
		fwrite("SYKG", 1, 4, fp);
	}
	~Dump() { if (fp) fclose(fp); }
	void rec(const std::string &name, uint8_t dt, const void *p, uint64_t n, size_t esz) {
		uint32_t nl = (uint32_t)name.size();
		fwrite(&nl, 4, 1, fp);
		fwrite(name.data(), 1, nl, fp);
		fwrite(&dt, 1, 1, fp);
		fwrite(&n, 8, 1, fp);
		if (n) fwrite(p, esz, n, fp);
	}
	void i32(const std::string &name, const std::vector<int> &v) { rec(name, 0, v.data(), v.size(), 4); }
	void f64(const std::string &name, const std::vector<double> &v) { rec(name, 1, v.data(), v.size(), 8); }
	void scalar_i(const std::string &name, int x) { std::vector<int> v(1, x); i32(name, v); }
	void scalar_d(const std::string &name, double x) { std::vector<double> v(1, x); f64(name, v); }
};

// ---------------------------------------------------------------------------
// Problem description
struct Case {
	std::string name;
	int nroot[3] = {1, 1, 1};
	int nb = 4;
	int minlevel = 1, maxlevel = 1;
	double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
	// refinement: blocks whose corners straddle the sphere |x-c| = r
	double rc[3] = {0, 0, 0}, rr = 0;
	// physical BC code per face (<= -20), and math BC per code
	int bc_code[6] = {-20, -20, -20, -20, -20, -20};
	int bc_math_m20 = Neumann, bc_math_m21 = Neumann; // math BC for codes -20 / -21
	// IB: solid sphere center/radius, 0 radius = none
	double ibc[3] = {0, 0, 0}, ibr = 0;
	int ib_binary = 0; // use setIBFracByLS instead of fractional injection
	// coefficient B = 1 + bamp*sin(2pi x)cos(2pi y)
	double bamp = 0;
	// solve settings
	int do_solve = 0;
	double tol_rel = 1e-10, tol_abs = 0;
	int rhs_gauss = 0; // 8 gaussians (config-1 style) instead of random
	int do_ops = 0;    // dump operator-level tests
	uint64_t seed = 12345;
	int cap = 20000;   // block capacity (every TreeData allocates for this many blocks)
	// bottom BiCGSTAB tolerances of the full solve (the reference defaults
	// 1e-6 / 1e-6 stall the outer solve on 16^d-cell blocks: the absolute
	// bottom tolerance weakens the preconditioner as the residual falls)
	double bot_tol_rel = 1e-6, bot_tol_abs = 1e-6;
	int ngrow = 1;     // tree ghost layers (centered-linear prolongation needs 2)
};

// the reference's AmrTree::init with a chosen block capacity (the reference
// hard-codes 40000 blocks; every TreeData allocates for that many)
static void tree_alloc(AmrTree &t, int cap) {
	t.maxBlockNum = cap;
	t.maxTreeBlockNum = cap;
	t.numBlocks = 0;
	t.gridChanged = 0;
	t.blocks = new AmrTreeNode[cap];
	t.refineFlag = new int[cap];
	t.coarsenFlag = new int[cap];
	t.newChildFlag = new int[cap];
	t.stayFlag = new int[cap];
	t.surrBlocks = new SurroundingBlocks[cap];
	for (int i = 0; i < cap; i++) {
		t.blocks[i].setUnused();
		t.refineFlag[i] = 0;
		t.coarsenFlag[i] = 0;
		t.newChildFlag[i] = 0;
		t.stayFlag[i] = 1;
		t.surrBlocks[i].setUnused();
	}
	t.levels.resize(t.maxAmrLevel + 1);
	for (int l = 0; l <= t.maxAmrLevel; l++) {
		t.levels[l].level = l;
		t.levels[l].clear();
	}
}

static double sphere_ls(const Case &c, const double x[3]) {
	double d2 = 0;
	for (int d = 0; d < NDIM; d++) d2 += (x[d] - c.rc[d]) * (x[d] - c.rc[d]);
	return sqrt(d2) - c.rr;
}

static bool block_straddles(const Case &c, const AmrTreeNode &b) {
	int nin = 0, nout = 0;
	for (int corner = 0; corner < (1 << NDIM); corner++) {
		double x[3] = {0, 0, 0};
		for (int d = 0; d < NDIM; d++)
			x[d] = ((corner >> d) & 1) ? b.boundBox.vhi(d) : b.boundBox.vlo(d);
		if (sphere_ls(c, x) < 0) nin++; else nout++;
	}
	return nin > 0 && nout > 0;
}

static void build_tree(const Case &c, AmrTree &tree, int cap) {
	tree.minAmrLevel = c.minlevel;
	tree.maxAmrLevel = c.maxlevel;
	IndexBox vbox(Vector3i::VecMake(0, 0, 0),
		Vector3i::VecMake(c.nb - 1, c.nb - 1, NDIM == 3 ? c.nb - 1 : 0));
	tree.blockValidIndex = vbox;
	tree.blockGrownIndex = IndexBox::Extend(vbox, c.ngrow);
	tree.blockNumGrow = c.ngrow;
	tree_alloc(tree, cap);

	RealBox pbox(c.lo, c.hi);
	bool periodic[6] = {false, false, false, false, false, false};
	tree.initUniformRootLevel(Vector3i::VecMake(c.nroot[0], c.nroot[1], c.nroot[2]),
		pbox, c.bc_code, periodic);
	tree.initRefineToMinLevel();

	for (int level = 1; level < c.maxlevel; level++) {
		for (int i = 0; i < tree.numBlocks; i++) {
			if (tree[i].getLevel() == level && tree[i].isLeaf() && block_straddles(c, tree[i]))
				tree.refineFlag[i] = 1;
		}
		tree.regrid();
	}
}

// ---------------------------------------------------------------------------
// field helpers: valid cells, block-major, i fastest
static int cells_per_block(const AmrTree &t) { return t.validBlockCellBox().stride(); }

static std::vector<double> get_cell(const TreeData &td, int comp, const std::vector<int> &blocks) {
	const IndexBox &vb = td.validBox();
	std::vector<double> out;
	out.reserve(blocks.size() * vb.stride());
	for (int b : blocks) {
		const DoubleBlockData &d = td[b];
		for (int k = vb.klo(); k <= vb.khi(); k++)
			for (int j = vb.jlo(); j <= vb.jhi(); j++)
				for (int i = vb.ilo(); i <= vb.ihi(); i++) out.push_back(d(i, j, k, comp));
	}
	return out;
}
static void set_cell(TreeData &td, int comp, const std::vector<int> &blocks, const std::vector<double> &v) {
	const IndexBox &vb = td.validBox();
	size_t p = 0;
	for (int b : blocks) {
		DoubleBlockData &d = td[b];
		for (int k = vb.klo(); k <= vb.khi(); k++)
			for (int j = vb.jlo(); j <= vb.jhi(); j++)
				for (int i = vb.ilo(); i <= vb.ihi(); i++) d(i, j, k, comp) = v[p++];
	}
}
static std::vector<int> all_blocks(const AmrTree &t) {
	std::vector<int> v(t.numBlocks);
	for (int i = 0; i < t.numBlocks; i++) v[i] = i;
	return v;
}
// seeded inputs that tests/golden_io.py regenerates bit-for-bit:
// value[i] = 2 * (splitmix64(seed*2^32 + tag*2^20 + i) >> 11) * 2^-53 - 1
static inline uint64_t splitmix64(uint64_t x) {
	uint64_t z = x + 0x9E3779B97F4A7C15ULL;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}
static uint64_t g_seed = 0;
static std::vector<double> rand_vec(uint64_t tag, size_t n) {
	std::vector<double> v(n);
	const uint64_t base = (g_seed << 32) + (tag << 20);
	for (size_t i = 0; i < n; i++) {
		uint64_t z = splitmix64(base + i);
		v[i] = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
	}
	return v;
}

// cell / face centre coordinates
static void cell_x(const AmrTree &t, int b, int i, int j, int k, double x[3]) {
	Vector3d dx = t.getBlockCellSize(b);
	const RealBox &bb = t[b].boundBox;
	int ijk[3] = {i, j, k};
	for (int d = 0; d < 3; d++) x[d] = 0;
	for (int d = 0; d < NDIM; d++) x[d] = bb.vlo(d) + (ijk[d] + 0.5) * dx(d);
}

// ---------------------------------------------------------------------------
// MacSolver subclass: gives the dump access to the solver's protected fields
// (IB fractions, coefficients) -- the reference's own extension point for
// fractional IB fractions (the public API only produces binary ones).
class ProbeSolver : public MacSolver {
public:
	explicit ProbeSolver(const AmrTree &t) : MacSolver(t) {}
	TreeData &volfrac() { return *m_ib_volfrac; }
	TreeData &areafrac(int d) { return *m_ib_areafrac[d]; }
	TreeData &bcoef(int d) { return *m_bcoef[d]; }
	const BlockBCRecord &bcrec(int b) const { return m_bc_rec[b]; }
	void setBottomTolerance(double rel, double abs) { m_mg_bot_tol_rel = rel; m_mg_bot_tol_abs = abs; }

	// fractional IB injection: leaf values are written directly, then the same
	// c/f AVG sync + AVG restriction that calcIBFracByLS performs
	void injectIBFrac(const Case &c) {
		const AmrTree &tree = getTree();
		int finest = tree.currentFinestLevel();
		const MGLevelTower &tower = getTower(finest);
		const IndexBox &vb = tree.validBlockCellBox();
		for (int ig = 0; ig < tower.numLevelBlock; ig++) {
			int b = tower[ig];
			Vector3d dx = tree.getBlockCellSize(b);
			double h = dx.x;
			DoubleBlockData &vf = (*m_ib_volfrac)[b];
			for (int k = vb.klo(); k <= vb.khi(); k++)
				for (int j = vb.jlo(); j <= vb.jhi(); j++)
					for (int i = vb.ilo(); i <= vb.ihi(); i++) {
						double x[3];
						cell_x(tree, b, i, j, k, x);
						vf(i, j, k, 0) = frac_of(c, x, h);
					}
			for (int d = 0; d < NDIM; d++) {
				DoubleBlockData &af = (*m_ib_areafrac[d])[b];
				int ii = d == 0, jj = d == 1, kk = d == 2;
				for (int k = vb.klo(); k <= vb.khi() + kk; k++)
					for (int j = vb.jlo(); j <= vb.jhi() + jj; j++)
						for (int i = vb.ilo(); i <= vb.ihi() + ii; i++) {
							double x[3];
							cell_x(tree, b, i, j, k, x);
							x[d] -= 0.5 * dx(d);
							af(i, j, k, 0) = frac_of(c, x, h);
						}
			}
		}
		for (int l = finest; l >= 2; l--)
			for (int d = 0; d < NDIM; d++)
				tower.syncSubLevelCrseFineFlux(l, l - 1, d, *m_ib_areafrac[d], 0, MGLevelTower::FLUX_SYNC_AVG);
		{
			FillPatch fill(const_cast<AmrTree &>(tree), *m_ib_volfrac);
			fill.setRestriction(0, InterpPatch::RESTRICT_AVERAGE);
			for (int l = finest - 1; l >= 1; l--) fill.restrictLevel(l, 0, 1);
		}
		for (int d = 0; d < NDIM; d++) {
			FillPatch fill(const_cast<AmrTree &>(tree), *m_ib_areafrac[d]);
			fill.setRestriction(0, InterpPatch::RESTRICT_AVERAGE);
			for (int l = finest - 1; l >= 1; l--) fill.restrictLevel(l, 0, 1);
		}
	}
	static double frac_of(const Case &c, const double x[3], double h) {
		double d2 = 0;
		for (int d = 0; d < NDIM; d++) d2 += (x[d] - c.ibc[d]) * (x[d] - c.ibc[d]);
		double s = (sqrt(d2) - c.ibr) / h + 0.5; // fluid outside the solid sphere
		if (s < 0) s = 0;
		if (s > 1) s = 1;
		// quantise so that fractions are exact binary fractions
		return floor(s * 64.0) / 64.0;
	}
};

// ---------------------------------------------------------------------------
static void dump_tree(Dump &D, const AmrTree &t) {
	const int n = t.numBlocks;
	std::vector<int> level(n), nb6(n * 6), ch8(n * 8), par(n), wc(n), nt(n), nt2(n * 6);
	std::vector<int> sb(n * 27), st(n * 27), sr(n * 27);
	std::vector<double> lo(n * 3), hi(n * 3), len(n * 3), cen(n * 3);
	for (int i = 0; i < n; i++) {
		const AmrTreeNode &b = t[i];
		level[i] = b.refineLevel;
		for (int f = 0; f < 6; f++) { nb6[i * 6 + f] = b.neighbor[f]; nt2[i * 6 + f] = b.nodeType2[f]; }
		for (int c = 0; c < 8; c++) ch8[i * 8 + c] = b.child[c];
		par[i] = b.parent;
		wc[i] = b.whichChild;
		nt[i] = b.nodeType;
		for (int d = 0; d < 3; d++) {
			lo[i * 3 + d] = b.boundBox.vlo(d);
			hi[i * 3 + d] = b.boundBox.vhi(d);
			len[i * 3 + d] = b.blockLength(d);
			cen[i * 3 + d] = b.blockCenter(d);
		}
		// surrounding tables in SurroundingIndex order (i fastest)
		for (int kk = 0; kk < 3; kk++)
			for (int jj = 0; jj < 3; jj++)
				for (int ii = 0; ii < 3; ii++) {
					int s = ii + 3 * jj + 9 * kk;
					sb[i * 27 + s] = t.surrBlocks[i].blocks[ii][jj][kk];
					st[i * 27 + s] = t.surrBlocks[i].types[ii][jj][kk];
					sr[i * 27 + s] = t.surrBlocks[i].bcrefs[ii][jj][kk];
				}
	}
	D.scalar_i("ndim", NDIM);
	D.scalar_i("nb", t.validBlockCellBox().size(0));
	D.scalar_i("num_blocks", n);
	D.scalar_i("min_level", t.minAmrLevel);
	D.scalar_i("max_level", t.maxAmrLevel);
	D.scalar_i("finest_level", t.currentFinestLevel());
	D.i32("level", level);
	D.i32("neighbor", nb6);
	D.i32("child", ch8);
	D.i32("parent", par);
	D.i32("which_child", wc);
	D.i32("node_type", nt);
	D.i32("node_type2", nt2);
	D.f64("block_lo", lo);
	D.f64("block_hi", hi);
	D.f64("block_len", len);
	D.f64("block_center", cen);
	D.i32("surr_blocks", sb);
	D.i32("surr_types", st);
	D.i32("surr_bcrefs", sr);
	for (int l = 1; l <= t.maxAmrLevel; l++) {
		D.i32("tree_level_" + std::to_string(l), t.levels[l].levelBlock);
	}
}

static void dump_towers(Dump &D, MacSolver &S, const AmrTree &t) {
	const int NCF = ChildIndex::NumChildOnFace;
	for (int L = 1; L <= t.maxAmrLevel; L++) {
		const MGLevelTower &tw = S.getTower(L);
		std::string p = "tower_" + std::to_string(L) + "_";
		std::vector<int> blocks(tw.levelBlock.begin(), tw.levelBlock.begin() + tw.numLevelBlock);
		D.i32(p + "blocks", blocks);
		std::vector<int> be;
		if (tw.numLevelBlock > 0)
			for (int l = 1; l <= L; l++) { be.push_back(tw.begin(l)); be.push_back(tw.end(l)); }
		D.i32(p + "begin_end", be);
		// face registers: per tower block, per face:
		// type, neigh, fine_crse_offset[3], crse_fine_neigh[4]
		// (crse_fine_offset / crse_fine_subbox are the ChildIndex tables below)
		std::vector<int> fr;
		for (int b : blocks) {
			for (int f = 0; f < FaceIndex::NumFace; f++) {
				const BlockFaceRegister &r = tw.getFaceReg(b, f);
				fr.push_back(r.face_type);
				fr.push_back(r.face_neigh);
				bool fc = r.face_type == FACE_FINE_CRSE, cf = r.face_type == FACE_CRSE_FINE;
				for (int d = 0; d < 3; d++) fr.push_back(fc ? r.fine_crse_offset(d) : 0);
				for (int q = 0; q < 4; q++) fr.push_back(cf && q < NCF ? r.crse_fine_neigh[q] : -1);
				if (cf) {
					// the per-child offsets/sub-boxes must be the ChildIndex ones
					int cnt = 0;
					for (int ch = 0; ch < ChildIndex::NumChild; ch++) {
						ChildIndex ci(ch);
						if (!ci.hasFaceBoundary(FaceIndex(f).opposite())) continue;
						Vector3i off = ChildIndex::ChildIndexOffset(t.validBlockCellBox(), ci);
						IndexBox sb = ChildIndex::ChildSubIndexRange(t.validBlockCellBox(), ci);
						if (!(off == r.crse_fine_offset[cnt]) || !(sb == r.crse_fine_subbox[cnt])) {
							fprintf(stderr, "unexpected crse_fine offset table\n");
							exit(4);
						}
						cnt++;
					}
				}
			}
		}
		D.i32(p + "face_regs", fr);
	}
}

static std::vector<double> get_face(const TreeData &td, const std::vector<int> &blocks) {
	return get_cell(td, 0, blocks); // validBox of face data is already staggered
}

// 2D fixtures keep every tower; 3D ones keep towers 1, finest-1, finest
static bool dump_tower(int L, int finest) {
	return NDIM == 2 || L == 1 || L >= finest - 1;
}

// iterations of the mg_solve / relax_solve dumps (tests/golden_io.py: MG_ITERS, RELAX_ITERS)
static const int kMgIters = 6, kRelaxIters = 25;

// ---------------------------------------------------------------------------
static void run_case(const Case &c, const char *outdir, int cap) {
	std::string path = std::string(outdir) + "/" + c.name + ".bin";
	Dump D(path.c_str());
	std::mt19937_64 rng(c.seed);
	g_seed = c.seed;

	AmrTree tree;
	build_tree(c, tree, cap);
	const int finest = tree.currentFinestLevel();
	fprintf(stderr, "[%s] blocks=%d finest=%d\n", c.name.c_str(), tree.numBlocks, finest);
	// reference hazard: level-1 leaves alias the bottom solve's buffers
	for (int i = 0; i < tree.numBlocks; i++)
		if (tree[i].getLevel() == 1 && tree[i].isLeaf() && finest > 1) {
			fprintf(stderr, "[%s] level-1 leaf present; refusing (bottom-solve aliasing)\n", c.name.c_str());
			exit(3);
		}
	dump_tree(D, tree);

	std::unique_ptr<ProbeSolver> S(new ProbeSolver(tree));
	S->prepareSolver();
	dump_towers(D, *S, tree);

	const std::vector<int> ALL = all_blocks(tree);
	const int ncell = cells_per_block(tree);

	// BC register: code -20 -> bc_math_m20, -21 -> bc_math_m21 (values 0)
	BCRegister bcreg;
	for (int s = 0; s < SurroundingIndex::NumSurr; s++) {
		SurroundingIndex si(s);
		bcreg.setBCMap(si, -20, c.bc_math_m20);
		bcreg.setBCMap(si, -21, c.bc_math_m21);
	}
	S->setBC(bcreg);
	{
		std::vector<int> bct(tree.numBlocks * 6);
		for (int b = 0; b < tree.numBlocks; b++)
			for (int f = 0; f < 6; f++) bct[b * 6 + f] = f < FaceIndex::NumFace ? S->bcrec(b).type(f) : -1;
		D.i32("bc_type", bct);
	}

	const MGLevelTower &TF = S->getTower(finest);
	std::vector<int> LEAF(TF.levelBlock.begin(), TF.levelBlock.begin() + TF.numLevelBlock);

	// IB fractions
	if (c.ibr > 0) {
		if (c.ib_binary) {
			// level set with ghosts, evaluated analytically (binary fractions)
			std::unique_ptr<TreeData> ls(TreeData::CreateCellData(tree, 1, 1));
			const IndexBox gb = IndexBox::Extend(tree.validBlockCellBox(), 1);
			for (int b = 0; b < tree.numBlocks; b++) {
				DoubleBlockData &d = (*ls)[b];
				for (int k = gb.klo(); k <= gb.khi(); k++)
					for (int j = gb.jlo(); j <= gb.jhi(); j++)
						for (int i = gb.ilo(); i <= gb.ihi(); i++) {
							double x[3];
							cell_x(tree, b, i, j, k, x);
							double d2 = 0;
							for (int q = 0; q < NDIM; q++) d2 += (x[q] - c.ibc[q]) * (x[q] - c.ibc[q]);
							d(i, j, k, 0) = sqrt(d2) - c.ibr;
						}
			}
			// dump the LS exactly as given (grown box, ghosts included)
			std::vector<double> lsv;
			for (int b = 0; b < tree.numBlocks; b++) {
				const DoubleBlockData &d = (*ls)[b];
				for (int k = gb.klo(); k <= gb.khi(); k++)
					for (int j = gb.jlo(); j <= gb.jhi(); j++)
						for (int i = gb.ilo(); i <= gb.ihi(); i++) lsv.push_back(d(i, j, k, 0));
			}
			D.f64("in_ls_grown", lsv);
			S->setIBFracByLS(*ls, 0);
		} else {
			S->injectIBFrac(c);
		}
	}
	// the leaf values the product receives (before sync/restrict) are
	// recomputable; the dump holds the final synced/restricted fields
	if (c.ibr > 0) {
		D.f64("vf", get_cell(S->volfrac(), 0, ALL));
		for (int d = 0; d < NDIM; d++) D.f64("af" + std::to_string(d), get_face(S->areafrac(d), ALL));
	}

	// variable B coefficient on leaf faces via the public setter
	if (c.bamp != 0) {
		std::vector<TreeData *> bd;
		std::vector<std::unique_ptr<TreeData>> own;
		for (int d = 0; d < NDIM; d++) {
			own.emplace_back(TreeData::CreateFaceData(tree, d, 1, 0));
			TreeData &fd = *own.back();
			fd.setValue(-777.0);
			const IndexBox &fb = fd.validBox();
			for (int b : LEAF) {
				Vector3d dx = tree.getBlockCellSize(b);
				DoubleBlockData &dd = fd[b];
				for (int k = fb.klo(); k <= fb.khi(); k++)
					for (int j = fb.jlo(); j <= fb.jhi(); j++)
						for (int i = fb.ilo(); i <= fb.ihi(); i++) {
							double x[3];
							cell_x(tree, b, i, j, k, x);
							x[d] -= 0.5 * dx(d);
							double v = 1.0 + c.bamp * sin(2 * M_PI * x[0]) * cos(2 * M_PI * x[1]);
							dd(i, j, k, 0) = floor(v * 1024.0) / 1024.0;
						}
			}
			D.f64("in_b" + std::to_string(d), get_face(fd, ALL));
			bd.push_back(&fd);
		}
		S->setCoefB(bd, 0);
	}
	if (c.bamp != 0)
		for (int d = 0; d < NDIM; d++) D.f64("bcoef" + std::to_string(d), get_face(S->bcoef(d), ALL));

	TreeData &buf = S->getDataBuf();

	if (c.do_ops) {
		// --- operator on every tower: out = L(x) ---
		std::vector<double> x = rand_vec(1, (size_t)tree.numBlocks * ncell);
		for (int L = 1; L <= finest; L++) {
			if (!dump_tower(L, finest)) continue;
			set_cell(buf, MacSolver::COMP_CG_P, ALL, x);
			TreeData::SetValue(buf, 0.0, MacSolver::COMP_CG_V, 1, 0);
			S->mg_apply_level(L, buf, buf, MacSolver::COMP_CG_V, MacSolver::COMP_CG_P);
			const MGLevelTower &tw = S->getTower(L);
			std::vector<int> tb(tw.levelBlock.begin(), tw.levelBlock.begin() + tw.numLevelBlock);
			D.f64("op_apply_" + std::to_string(L), get_cell(buf, MacSolver::COMP_CG_V, tb));
		}
		// residual at finest: r = rhs - L(x)
		{
			std::vector<double> rhs = rand_vec(2, (size_t)tree.numBlocks * ncell);
			set_cell(buf, MacSolver::COMP_CG_P, ALL, x);
			set_cell(buf, MacSolver::COMP_CG_S, ALL, rhs);
			S->mg_residual_level(finest, buf, buf, buf, MacSolver::COMP_CG_T, MacSolver::COMP_CG_P, MacSolver::COMP_CG_S);
			D.f64("op_resid", get_cell(buf, MacSolver::COMP_CG_T, LEAF));
		}
		// --- smoother: one mg_smooth_level per tower ---
		{
			std::vector<double> corr = rand_vec(3, (size_t)tree.numBlocks * ncell);
			std::vector<double> res = rand_vec(4, (size_t)tree.numBlocks * ncell);
			for (int L = 1; L <= finest; L++) {
				if (!dump_tower(L, finest)) continue;
				set_cell(buf, MacSolver::COMP_BUF_CORR, ALL, corr);
				set_cell(buf, MacSolver::COMP_BUF_RESID, ALL, res);
				S->mg_smooth_level(L, buf, buf, MacSolver::COMP_BUF_CORR, MacSolver::COMP_BUF_RESID);
				// only tower blocks change; the others keep sm_corr0
				const MGLevelTower &tw = S->getTower(L);
				std::vector<int> tb(tw.levelBlock.begin(), tw.levelBlock.begin() + tw.numLevelBlock);
				D.f64("sm_out_" + std::to_string(L), get_cell(buf, MacSolver::COMP_BUF_CORR, tb));
			}
		}
		// --- restriction sweep finest..2 (volume weighted) ---
		{
			std::vector<double> res = rand_vec(5, (size_t)tree.numBlocks * ncell);
			set_cell(buf, MacSolver::COMP_BUF_RESID, ALL, res);
			for (int l = finest; l >= 2; l--) S->mg_restict_wgt(l - 1, buf, MacSolver::COMP_BUF_RESID);
			D.f64("rs_out", get_cell(buf, MacSolver::COMP_BUF_RESID, ALL));
		}
		// --- prolongation sweep 2..finest (masked injection) ---
		{
			std::vector<double> cr = rand_vec(6, (size_t)tree.numBlocks * ncell);
			set_cell(buf, MacSolver::COMP_BUF_CORR, ALL, cr);
			for (int l = 2; l <= finest; l++) S->mg_prolong_wgt(l, buf, MacSolver::COMP_BUF_CORR);
			D.f64("pr_out", get_cell(buf, MacSolver::COMP_BUF_CORR, ALL));
		}
		// --- face flux -B grad(phi) after a fill (mg_flux_level) ---
		{
			std::vector<double> phi = rand_vec(7, (size_t)tree.numBlocks * ncell);
			for (int d = 0; d < NDIM; d++) {
				std::unique_ptr<TreeData> fl(TreeData::CreateFaceData(tree, d, 1, 0));
				fl->setValue(0.0);
				set_cell(buf, MacSolver::COMP_CG_P, ALL, phi);
				S->mg_flux_level(finest, d, *fl, buf, 0, MacSolver::COMP_CG_P);
				D.f64("fx_out" + std::to_string(d), get_face(*fl, LEAF));
			}
		}
		// --- one V-cycle preconditioner application: phat = M^-1 p ---
		{
			std::vector<double> p = rand_vec(8, (size_t)tree.numBlocks * ncell);
			if (c.bc_math_m20 == Neumann && c.bc_math_m21 == Neumann) {
				// singular (all-Neumann) operator: make p compatible so that the
				// bottom BiCGSTAB of the V-cycle has a solution
				const std::vector<double> vf = get_cell(S->volfrac(), 0, ALL);
				double s = 0, v = 0;
				for (int b : LEAF) {
					double dv = tree.getBlockCellVolume(b);
					for (int q = 0; q < ncell; q++) {
						double w = vf[(size_t)b * ncell + q];
						if (w > 0) { s += p[(size_t)b * ncell + q] * dv * w; v += dv * w; }
					}
				}
				for (int b : LEAF) for (int q = 0; q < ncell; q++) p[(size_t)b * ncell + q] -= s / v;
			}
			D.f64("vc_p", p);
			TreeData::SetValue(buf, 0.0, 0, MacSolver::NUM_COMP_BUF, 1);
			set_cell(buf, MacSolver::COMP_CG_P, ALL, p);
			S->mg_precond_level(finest, buf, buf, MacSolver::COMP_CG_PHAT, MacSolver::COMP_CG_P);
			D.f64("vc_phat", get_cell(buf, MacSolver::COMP_CG_PHAT, LEAF));
		}
		// --- Dirichlet lift of the RHS (fixBC), BC values held in phi's ghosts ---
		{
			std::unique_ptr<TreeData> phi(TreeData::CreateCellData(tree, 1, 1));
			std::unique_ptr<TreeData> rhs(TreeData::CreateCellData(tree, 1, 1));
			const IndexBox gb = IndexBox::Extend(tree.validBlockCellBox(), 1);
			std::vector<double> pg = rand_vec(9, (size_t)tree.numBlocks * gb.stride());
			std::vector<double> r0 = rand_vec(10, (size_t)tree.numBlocks * ncell);
			size_t q = 0;
			for (int b = 0; b < tree.numBlocks; b++) {
				DoubleBlockData &d = (*phi)[b];
				for (int k = gb.klo(); k <= gb.khi(); k++)
					for (int j = gb.jlo(); j <= gb.jhi(); j++)
						for (int i = gb.ilo(); i <= gb.ihi(); i++) d(i, j, k, 0) = pg[q++];
			}
			set_cell(*rhs, 0, ALL, r0);
			S->fixBC(*phi, *rhs, 0, 0);
			D.f64("bc_rhs", get_cell(*rhs, 0, ALL));
		}
	}

	if (c.do_solve) {
		// right-hand side: config-1 style Gaussians, or random; Neumann-only
		// problems get the volume-weighted mean (over vf>0 cells) removed
		std::vector<double> f((size_t)tree.numBlocks * ncell, 0.0);
		if (c.rhs_gauss) {
			std::normal_distribution<double> N01(0.0, 1.0);
			std::uniform_real_distribution<double> U(0.1, 0.9);
			double amp[8], cx[8][3];
			for (int g = 0; g < 8; g++) {
				amp[g] = N01(rng);
				for (int d = 0; d < 3; d++) cx[g][d] = d < NDIM ? U(rng) : 0.0;
			}
			const IndexBox &vb = tree.validBlockCellBox();
			for (int b : LEAF) {
				size_t p = (size_t)b * ncell;
				for (int k = vb.klo(); k <= vb.khi(); k++)
					for (int j = vb.jlo(); j <= vb.jhi(); j++)
						for (int i = vb.ilo(); i <= vb.ihi(); i++) {
							double x[3];
							cell_x(tree, b, i, j, k, x);
							double s = 0;
							for (int g = 0; g < 8; g++) {
								double r2 = 0;
								for (int d = 0; d < NDIM; d++) r2 += (x[d] - cx[g][d]) * (x[d] - cx[g][d]);
								s += amp[g] * exp(-r2 / (2 * 0.05 * 0.05));
							}
							f[p++] = s;
						}
			}
		} else {
			std::vector<double> r = rand_vec(11, f.size());
			for (int b : LEAF) for (int q = 0; q < ncell; q++) f[(size_t)b * ncell + q] = r[(size_t)b * ncell + q];
		}
		bool all_neumann = c.bc_math_m20 == Neumann && c.bc_math_m21 == Neumann;
		if (all_neumann) {
			const std::vector<double> vf = get_cell(S->volfrac(), 0, ALL);
			double s = 0, v = 0;
			for (int b : LEAF) {
				double dv = tree.getBlockCellVolume(b);
				for (int q = 0; q < ncell; q++) {
					double w = vf[(size_t)b * ncell + q];
					if (w > 0) { s += f[(size_t)b * ncell + q] * dv * w; v += dv * w; }
				}
			}
			for (int b : LEAF) for (int q = 0; q < ncell; q++) f[(size_t)b * ncell + q] -= s / v;
		}
		// the reference solves -div(B grad phi) = rhs: feed rhs = -f
		for (auto &x : f) x = -x;
		D.f64("sv_rhs", f);
		std::unique_ptr<TreeData> ud(TreeData::CreateCellData(tree, 1, 1));
		set_cell(*ud, 0, ALL, f);
		S->setRhs(*ud, 0);
		S->setZeroSol();
		S->setTolerance(c.tol_rel, c.tol_abs);
		S->setBottomTolerance(c.bot_tol_rel, c.bot_tol_abs);
		D.scalar_d("sv_bot_tol_rel", c.bot_tol_rel);
		D.scalar_d("sv_bot_tol_abs", c.bot_tol_abs);
		S->setCGUseMGPrecond(1);
		S->setVerbose(1);
		int stat = S->cg_solve();
		S->getSol(*ud, 0);
		D.scalar_i("sv_stat", stat);
		D.f64("sv_sol", get_cell(*ud, 0, LEAF));
		// true residual of the returned solution
		TreeData::SetValue(buf, 0.0, MacSolver::COMP_CG_T, 1, 1);
		set_cell(buf, MacSolver::COMP_CG_P, ALL, get_cell(*ud, 0, ALL));
		set_cell(buf, MacSolver::COMP_CG_S, ALL, f);
		S->mg_residual_level(finest, buf, buf, buf, MacSolver::COMP_CG_T, MacSolver::COMP_CG_P, MacSolver::COMP_CG_S);
		double rn = S->mg_norm_level(finest, buf, MacSolver::COMP_CG_T);
		set_cell(buf, MacSolver::COMP_CG_T, ALL, f);
		double bn = S->mg_norm_level(finest, buf, MacSolver::COMP_CG_T);
		D.scalar_d("sv_true_resid_inf", rn);
		D.scalar_d("sv_rhs_inf", bn);
		fprintf(stderr, "[%s] solve stat=%d |r|inf=%.3e |b|inf=%.3e\n", c.name.c_str(), stat, rn, bn);
		// the other two solvers of the public API on the same problem, a fixed
		// number of iterations each (the relative tolerance is out of reach)
		if (c.do_ops && !all_neumann) {
			std::unique_ptr<TreeData> rd(TreeData::CreateCellData(tree, 1, 1));
			set_cell(*rd, 0, ALL, f);
			S->setRhs(*rd, 0);
			S->setZeroSol();
			S->setTolerance(1e-30, 0.0);
			S->setMaxIteration(kMgIters);
			S->setVerbose(0);
			// the preconditioned cg_solve above left the fixed V-cycle count
			// of the preconditioner (1) set, which mg_solve would obey
			S->setMGFixedIter(0);
			S->mg_solve();
			S->getSol(*ud, 0);
			D.f64("mg_sol", get_cell(*ud, 0, LEAF));
			S->setZeroSol();
			S->setMaxIteration(kRelaxIters);
			S->relax_solve();
			S->getSol(*ud, 0);
			D.f64("rx_sol", get_cell(*ud, 0, LEAF));
		}
	}
}

// moving-circle regrid sequence (refine near the interface, coarsen away from
// it), tables dumped after every regrid -- exercises coarsenBlocks' packing
static void run_regrid_case(const char *outdir, const std::string &name) {
  std::string path = std::string(outdir) + "/" + name + ".bin";
  Dump D(path.c_str());
  Case c;
  c.name = name;
  c.nroot[0] = 3;
  c.nroot[1] = 2;
  c.hi[0] = 1.5;
  c.hi[1] = 1.0;
  if (NDIM == 3) c.hi[2] = 1.0;
  c.nb = 4;
  c.minlevel = 2;
  c.maxlevel = NDIM == 3 ? 4 : 6;
  c.rr = 0.22;
  AmrTree tree;
  c.rc[0] = 0.35;
  c.rc[1] = 0.45;
  c.rc[2] = 0.5;
  build_tree(c, tree, 20000);
  D.scalar_i("steps", 6);
  for (int step = 0; step < 6; step++) {
    c.rc[0] += 0.11;
    c.rc[1] += 0.03 * (step % 2 ? -1 : 1);
    for (int pass = 0; pass < c.maxlevel; pass++) {
      for (int i = 0; i < tree.numBlocks; i++) {
        tree.refineFlag[i] = 0;
        tree.coarsenFlag[i] = 0;
        if (!tree[i].isLeaf()) continue;
        const bool near = block_straddles(c, tree[i]);
        if (near && tree[i].getLevel() < c.maxlevel) tree.refineFlag[i] = 1;
        if (!near && tree[i].getLevel() > c.minlevel) tree.coarsenFlag[i] = 1;
      }
      tree.regrid();
    }
    std::vector<int> level(tree.numBlocks), nbr(tree.numBlocks * 6), ch(tree.numBlocks * 8), par(tree.numBlocks);
    std::vector<int> sb(tree.numBlocks * 27);
    for (int i = 0; i < tree.numBlocks; i++) {
      level[i] = tree[i].refineLevel;
      par[i] = tree[i].parent;
      for (int f = 0; f < 6; f++) nbr[i * 6 + f] = tree[i].neighbor[f];
      for (int q = 0; q < 8; q++) ch[i * 8 + q] = tree[i].child[q];
      for (int kk = 0; kk < 3; kk++)
        for (int jj = 0; jj < 3; jj++)
          for (int ii = 0; ii < 3; ii++) sb[i * 27 + ii + 3 * jj + 9 * kk] = tree.surrBlocks[i].blocks[ii][jj][kk];
    }
    const std::string p = "step_" + std::to_string(step) + "_";
    D.i32(p + "level", level);
    D.i32(p + "neighbor", nbr);
    D.i32(p + "child", ch);
    D.i32(p + "parent", par);
    D.i32(p + "surr_blocks", sb);
  }
  fprintf(stderr, "[%s] blocks=%d\n", name.c_str(), tree.numBlocks);
}

static void dump_tables(Dump &D, const std::string &p, const AmrTree &t) {
  const int n = t.numBlocks;
  std::vector<int> level(n), nbr(n * 6), ch(n * 8), par(n), wc(n), nt(n);
  for (int i = 0; i < n; i++) {
    level[i] = t[i].refineLevel;
    par[i] = t[i].parent;
    wc[i] = t[i].whichChild;
    nt[i] = t[i].nodeType;
    for (int f = 0; f < 6; f++) nbr[i * 6 + f] = t[i].neighbor[f];
    for (int q = 0; q < 8; q++) ch[i * 8 + q] = t[i].child[q];
  }
  D.scalar_i(p + "num_blocks", n);
  D.i32(p + "level", level);
  D.i32(p + "neighbor", nbr);
  D.i32(p + "child", ch);
  D.i32(p + "parent", par);
  D.i32(p + "which_child", wc);
  D.i32(p + "node_type", nt);
}

// A cell field carried across one regrid by the reference itself: the field
// (two ghost layers) is registered as the tree's state with centered-linear
// prolongation and average restriction (the pressure settings of
// src/Test6.h:618-631) and a BC register that uses every math BC kind with
// non-zero values; random leaf values are averaged down (restrictAll), one
// regrid refines near a moved circle and coarsens away from it, and
// AmrTree::initNewBlockDataAfterRegrid fills the new blocks.  The old and new
// tables and the field before and after are dumped.
static void run_transfer_case(const char *outdir, const std::string &name) {
  std::string path = std::string(outdir) + "/" + name + ".bin";
  Dump D(path.c_str());
  Case c;
  c.name = name;
  for (int d = 0; d < NDIM; d++) c.hi[d] = 1.0;
  c.nb = NDIM == 3 ? 4 : 8;
  c.minlevel = 2;
  c.maxlevel = NDIM == 3 ? 4 : 5;
  // refinement around a small interior circle (sphere); the regrid then
  // follows a larger one that crosses the x, y-hi (and z) sides, so that
  // new blocks appear beside the physical boundaries
  c.rc[0] = 0.41;
  c.rc[1] = 0.33;
  c.rc[2] = 0.45;
  c.rr = 0.26;
  c.ngrow = 2;
  c.seed = NDIM == 3 ? 8803 : 8802;
  g_seed = c.seed;
  AmrTree tree;
  build_tree(c, tree, 20000);
  std::unique_ptr<TreeData> u(TreeData::CreateCellData(tree, 1, 2));
  BCPatch bcp;
  bcp.defineByData(*u);
  // x-lo Dirichlet 0.75, x-hi SimpleFill -0.5, y-lo and y-hi Neumann, z-lo
  // Neumann, z-hi Dirichlet 1.5; edges and corners Neumann
  const int math[6] = {Dirichlet, SimpleFill, Neumann, Neumann, Neumann, Dirichlet};
  const double val[6] = {0.75, -0.5, 0.0, 0.0, 0.0, 1.5};
  BCRegister &reg = bcp.boundaryRegister(0);
  for (int s = 0; s < SurroundingIndex::NumSurr; s++) reg.setBCMap(SurroundingIndex(s), -20, Neumann);
  std::vector<int> bc_math;
  std::vector<double> bc_val;
  for (int f = 0; f < FaceIndex::NumFace; f++) {
    const SurroundingIndex si = SurroundingIndex::FaceSurrounding(FaceIndex(f));
    reg.setBCMap(si, -20, math[f]);
    reg.setBCVal(si, -20, val[f]);
    bc_math.push_back(math[f]);
    bc_val.push_back(val[f]);
  }
  D.scalar_i("ndim", NDIM);
  D.scalar_i("nb", c.nb);
  D.i32("bc_math", bc_math);
  D.f64("bc_val", bc_val);
  FillPatch fill(tree, *u);
  fill.setProlongation(0, InterpPatch::PROLONG_CENTERED_LINEAR);
  fill.setRestriction(0, InterpPatch::RESTRICT_AVERAGE);
  fill.setBC(bcp);
  TreeStateData st;
  st.new_data = u.get();
  st.fill_new_patch = &fill;
  st.bc_patch = &bcp;
  tree.treeStateData.push_back(st);

  dump_tables(D, "old_", tree);
  const int ncell = cells_per_block(tree);
  set_cell(*u, 0, all_blocks(tree), rand_vec(1, (size_t)tree.numBlocks * ncell));
  fill.restrictAll(0, 1);
  D.f64("old_x", get_cell(*u, 0, all_blocks(tree)));

  // the circle moves and grows; one regrid pass refines and coarsens
  c.rc[0] = 0.47;
  c.rc[1] = 0.71;
  c.rc[2] = 0.5;
  c.rr = 0.56;
  int nref = 0, ncrs = 0;
  for (int i = 0; i < tree.numBlocks; i++) {
    tree.refineFlag[i] = 0;
    tree.coarsenFlag[i] = 0;
    if (!tree[i].isLeaf()) continue;
    const bool near = block_straddles(c, tree[i]);
    if (near && tree[i].getLevel() < c.maxlevel) tree.refineFlag[i] = 1, nref++;
    if (!near && tree[i].getLevel() > c.minlevel) tree.coarsenFlag[i] = 1, ncrs++;
  }
  tree.regrid();
  tree.initNewBlockDataAfterRegrid();
  std::vector<int> nc(tree.numBlocks);
  int nnew = 0;
  for (int i = 0; i < tree.numBlocks; i++) nc[i] = tree.newChildFlag[i], nnew += nc[i];
  dump_tables(D, "new_", tree);
  D.i32("new_child_flag", nc);
  D.f64("new_x", get_cell(*u, 0, all_blocks(tree)));
  fprintf(stderr, "[%s] blocks=%d refine flags=%d coarsen flags=%d new blocks=%d\n", name.c_str(), tree.numBlocks,
          nref, ncrs, nnew);
}

// ---------------------------------------------------------------------------
static Case make_case(const std::string &name) {
	Case c;
	c.name = name;
	for (int d = 0; d < NDIM; d++) c.hi[d] = 1.0;
#if SAYAKA_SPACEDIM == 2
	if (name == "c1") {
		// 2D unit square, 4x4 roots of 8x8, levels 1..4 around r=0.25 circle
		c.nroot[0] = c.nroot[1] = 4;
		c.nb = 8; c.minlevel = 1; c.maxlevel = 4;
		c.rc[0] = 0.5; c.rc[1] = 0.5; c.rr = 0.25;
		c.do_solve = 1; c.rhs_gauss = 1; c.tol_rel = 1e-10;
		c.seed = 20251;
	} else if (name == "t2s") {
		// small 2D fixture: mixed Neumann (x) / Dirichlet (y) walls,
		// fractional IB disk, variable B
		c.nroot[0] = c.nroot[1] = 2;
		c.nb = 4; c.minlevel = 2; c.maxlevel = 5;
		c.rc[0] = 0.43; c.rc[1] = 0.56; c.rr = 0.3;
		c.bc_code[2] = c.bc_code[3] = -21;
		c.bc_math_m21 = Dirichlet;
		c.ibc[0] = 0.62; c.ibc[1] = 0.40; c.ibr = 0.12;
		c.bamp = 0.5;
		c.do_ops = 1; c.do_solve = 1; c.tol_rel = 1e-12;
		c.seed = 777;
	} else if (name == "t2b") {
		// binary IB from a level set + Neumann walls + variable B
		c.nroot[0] = 2; c.nroot[1] = 1; c.hi[0] = 2.0;
		c.nb = 8; c.minlevel = 2; c.maxlevel = 4;
		c.rc[0] = 1.1; c.rc[1] = 0.45; c.rr = 0.33;
		c.ibc[0] = 0.7; c.ibc[1] = 0.55; c.ibr = 0.15; c.ib_binary = 1;
		c.bamp = 0.25;
		c.do_ops = 1; c.do_solve = 1; c.tol_rel = 1e-11;
		c.seed = 4242;
	} else if (name == "n2") {
		// the benchmark block size (16x16): 4 levels around a circle,
		// Neumann x walls / Dirichlet y walls, fractional IB disk, variable B
		c.nroot[0] = c.nroot[1] = 2;
		c.nb = 16; c.minlevel = 2; c.maxlevel = 5;
		c.rc[0] = 0.45; c.rc[1] = 0.52; c.rr = 0.3;
		c.bc_code[2] = c.bc_code[3] = -21;
		c.bc_math_m21 = Dirichlet;
		c.ibc[0] = 0.58; c.ibc[1] = 0.41; c.ibr = 0.11;
		c.bamp = 0.5;
		c.do_ops = 1; c.do_solve = 1; c.tol_rel = 1e-10;
		c.seed = 1616;
		c.cap = 1500;
		c.bot_tol_rel = 1e-10; c.bot_tol_abs = 0.0;
	} else {
		fprintf(stderr, "unknown 2D case %s\n", name.c_str());
		exit(2);
	}
#else
	if (name == "t3s") {
		c.nb = 4; c.minlevel = 2; c.maxlevel = 4;
		c.rc[0] = 0.47; c.rc[1] = 0.52; c.rc[2] = 0.55; c.rr = 0.21;
		c.bc_code[4] = c.bc_code[5] = -21;
		c.bc_math_m21 = Dirichlet;
		c.ibc[0] = 0.6; c.ibc[1] = 0.45; c.ibc[2] = 0.5; c.ibr = 0.14;
		c.bamp = 0.5;
		c.do_ops = 1; c.do_solve = 1; c.tol_rel = 1e-11;
		c.seed = 99;
	} else if (name == "t3n") {
		// all-Neumann 3D, binary IB
		c.nb = 4; c.minlevel = 2; c.maxlevel = 4;
		c.rc[0] = 0.5; c.rc[1] = 0.5; c.rc[2] = 0.5; c.rr = 0.2;
		c.ibc[0] = 0.35; c.ibc[1] = 0.6; c.ibc[2] = 0.45; c.ibr = 0.12; c.ib_binary = 1;
		c.do_ops = 1; c.do_solve = 1; c.tol_rel = 1e-10;
		c.seed = 31337;
	} else if (name == "n3") {
		// the benchmark block size (16^3): levels 2-4 refined around a sphere
		// holding one corner of the level-3 grid (coarse/fine faces on the
		// finest tower), Neumann
		// walls with a Dirichlet top, fractional IB sphere, variable B
		c.nb = 16; c.minlevel = 2; c.maxlevel = 4;
		c.rc[0] = 0.47; c.rc[1] = 0.52; c.rc[2] = 0.55; c.rr = 0.16;
		c.bc_code[5] = -21;
		c.bc_math_m21 = Dirichlet;
		c.ibc[0] = 0.45; c.ibc[1] = 0.5; c.ibc[2] = 0.52; c.ibr = 0.06;
		c.bamp = 0.5;
		c.do_ops = 1; c.do_solve = 1; c.tol_rel = 1e-10;
		c.seed = 4096;
		c.cap = 400;
		c.bot_tol_rel = 1e-10; c.bot_tol_abs = 0.0;
	} else {
		fprintf(stderr, "unknown 3D case %s\n", name.c_str());
		exit(2);
	}
#endif
	return c;
}

int main(int argc, char **argv) {
	if (argc < 3) {
		fprintf(stderr, "usage: %s OUTDIR CASE [CASE...]\n", argv[0]);
		return 2;
	}
	for (int a = 2; a < argc; a++) {
		if (std::string(argv[a]).rfind("rg", 0) == 0) {
			run_regrid_case(argv[1], argv[a]);
			continue;
		}
		if (std::string(argv[a]).rfind("tf", 0) == 0) {
			run_transfer_case(argv[1], argv[a]);
			continue;
		}
		Case c = make_case(argv[a]);
		run_case(c, argv[1], c.cap);
	}
	return 0;
}
