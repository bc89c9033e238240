// Reference harness (test infrastructure, never shipped or measured as the product).
//
// Builds the reference's own solve path from its headers, unmodified, and writes
// what it computes to a directory of raw little-endian arrays:
//
//   gen   <dim> <n> <k> <outdir> [--smoothers pre,post] [--no-solve]
//         Mesh + HHO assembly + MultigridForHHO setup exactly as
//         Program_Diffusion_HHO<Dim>::Execute does (src/Program/Program_Diffusion_HHO.h:241-277),
//         through SolverFactory<Dim>::CreateSolver (src/Solver/SolverFactory.h:156-200)
//         with "-s fcgmg -cs s -cycle V,1,1". Dumps every level's A, P, the
//         right-hand side b, per-face geometry, then (unless --no-solve) the FCG
//         residual history captured through IterativeSolver::OnIterationEnd
//         (src/Solver/IterativeSolver.h:224-227) and the solution x.
//
//   genp  <dim> <n> <k> <outdir> [--coarse-solver ch|mg] [--p-cs minus1|minus2]
//         The same pipeline with the p-multigrid preconditioner ("-s fcg -p p_mg", P_MultigridForHHO
//         through SolverFactory.h:201-211, P_CS Minus2 and CoarsePolyDegree 1 as defaulted) and the
//         coarse solver "-cs ch" (Cholesky of the lowest degree) or "-cs mg" (one h-multigrid cycle
//         on it, SolverFactory.h:299-308). Dumps the p-levels' A and P (the natural injection),
//         then, with "-cs mg", the levels of that coarse multigrid below its finest one, numbered on
//         from the p-levels; the block size of every level; the history and x.
//
//   solve <dir> [--smoothers pre,post] [--krylov fcg|cg] [--cycle V|W|K] [--tol t] [--maxit m] [--omega w]
//         Reads a hierarchy (possibly re-ordered by the caller) from <dir>, feeds it
//         to the reference's own Multigrid / BlockGaussSeidel / EigenSparseCholesky /
//         FlexibleConjugateGradient classes through a Level subclass that only
//         supplies the given A and P (R = P^T as LevelForHHO::SetupRestriction,
//         src/Solver/Multigrid/MultigridForHHO/LevelForHHO.h:535-543), and writes
//         the residual history and x. This is how the reference block Gauss-Seidel
//         is run in a colour ordering.
//
// Built by oracle/Makefile from the sources under the reference checkout; outputs
// go to oracle/_ref/ only.
#include "ProgramArguments.h"
#include "Discretizations/DG/Diffusion_DG.h"
#include "TestCases/Diffusion/DiffTestCaseFactory.h"
#include "Mesher/InHouse/Square_CartesianMesh.h"
#include "Mesher/InHouse/Square_TriangularMesh.h"
#include "Mesher/InHouse/Cube_CartesianTetrahedralMesh.h"
#include "FunctionalBasis/FunctionalBasisFactory.h"
#include "Discretizations/HHO/Diffusion_HHO.h"
#include "Solver/SolverFactory.h"

#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

// ---------------------------------------------------------------------------
// Access to protected members through pointers-to-member (standard C++; no
// reference header is modified).
struct LevelPAccess : Level { using Level::P; using Level::R; };
struct MGFineAccess : Multigrid { using Multigrid::_fineLevel; };
struct PrecondAccess : SolverPreconditioner { using SolverPreconditioner::_solver; };

static SparseMatrix& LevelP(Level* l) { return l->*(&LevelPAccess::P); }
static Level* MGFine(Multigrid* mg) { return mg->*(&MGFineAccess::_fineLevel); }
static Solver* PrecondSolver(SolverPreconditioner& p) { return p.*(&PrecondAccess::_solver); }

// ---------------------------------------------------------------------------
// Raw array I/O
template <class T>
static void WriteArray(const std::string& path, const T* data, size_t n)
{
	FILE* f = fopen(path.c_str(), "wb");
	if (!f) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(2); }
	if (n && fwrite(data, sizeof(T), n, f) != n) { fprintf(stderr, "short write %s\n", path.c_str()); exit(2); }
	fclose(f);
}

template <class T>
static std::vector<T> ReadArray(const std::string& path)
{
	FILE* f = fopen(path.c_str(), "rb");
	if (!f) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(2); }
	fseek(f, 0, SEEK_END);
	long bytes = ftell(f);
	fseek(f, 0, SEEK_SET);
	std::vector<T> v(bytes / sizeof(T));
	if (!v.empty() && fread(v.data(), sizeof(T), v.size(), f) != v.size()) { fprintf(stderr, "short read %s\n", path.c_str()); exit(2); }
	fclose(f);
	return v;
}

static void DumpCSR(const std::string& prefix, SparseMatrix M)
{
	M.makeCompressed();
	int rows = (int)M.rows(), cols = (int)M.cols();
	int shape[2] = { rows, cols };
	WriteArray(prefix + "_shape.i32", shape, 2);
	WriteArray(prefix + "_rowptr.i32", M.outerIndexPtr(), (size_t)rows + 1);
	WriteArray(prefix + "_colidx.i32", M.innerIndexPtr(), (size_t)M.nonZeros());
	WriteArray(prefix + "_vals.f64", M.valuePtr(), (size_t)M.nonZeros());
}

static SparseMatrix LoadCSR(const std::string& prefix)
{
	auto shape = ReadArray<int>(prefix + "_shape.i32");
	auto rowptr = ReadArray<int>(prefix + "_rowptr.i32");
	auto colidx = ReadArray<int>(prefix + "_colidx.i32");
	auto vals = ReadArray<double>(prefix + "_vals.f64");
	std::vector<Eigen::Triplet<double>> t;
	t.reserve(vals.size());
	for (int i = 0; i < shape[0]; i++)
		for (int p = rowptr[i]; p < rowptr[i + 1]; p++)
			t.emplace_back(i, colidx[p], vals[p]);
	SparseMatrix M(shape[0], shape[1]);
	M.setFromTriplets(t.begin(), t.end());
	M.makeCompressed();
	return M;
}

static void WriteText(const std::string& path, const std::string& s)
{
	std::ofstream f(path);
	f << s;
}

static void ParseSmoothers(const std::string& s, std::string& pre, std::string& post)
{
	auto c = s.find(',');
	pre = s.substr(0, c);
	post = c == std::string::npos ? pre : s.substr(c + 1);
}

// ---------------------------------------------------------------------------
// gen: the reference pipeline end to end.
template <int D>
static int RunGen(int n, int k, const std::string& outdir, const std::string& pre, const std::string& post, bool solve,
                  const std::string& precond = "mg", const std::string& coarseSolver = "ch",
                  P_CoarsStgy pcs = P_CoarsStgy::Minus2)
{
	ProgramArguments args;
	args.Problem.Dimension = D;
	args.Problem.GeoCode = D == 2 ? "square" : "cube";
	args.Problem.TestCaseCode = args.Problem.GeoCode;
	args.Problem.BCCode = "d";
	args.Discretization.N = n;
	args.Discretization.Mesher = "inhouse";
	args.Discretization.MeshCode = D == 2 ? "stri" : "stetra";
	args.Discretization.PolyDegree = k + 1;
	// Defaults resolved by src/main.cpp:1703-1735 for non-Cartesian meshes.
	args.Discretization.ElemBasisCode = "monomials";
	args.Discretization.OrthogonalizeElemBasesCode = 1;
	args.Discretization.FaceBasisCode = D == 2 ? "legendre" : "monomials";
	args.Discretization.OrthogonalizeFaceBasesCode = D == 2 ? 0 : 1;
	args.Solver.SolverCode = "fcg";
	args.Solver.PreconditionerCode = precond;
	args.Solver.Tolerance = 1e-8;
	args.Solver.MaxIterations = 200;
	args.Solver.PrintIterationResults = false;
	args.Solver.MG.H_CS = H_CoarsStgy::StandardCoarsening;
	args.Solver.MG.GMG_H_Prolong = GMG_H_Prolongation::CellInterp_Trace;
	args.Solver.MG.PreSmootherCode = pre;
	args.Solver.MG.PostSmootherCode = post;
	args.Solver.MG.PreSmoothingIterations = 1;
	args.Solver.MG.PostSmoothingIterations = 1;
	args.Solver.MG.CoarseSolverCode = coarseSolver;
	args.Solver.MG.P_CS = pcs;
	args.Actions.LogAssembly = false;
	Utils::ProgramArgs = args;
	GaussLegendre::Init();

	DiffusionTestCase<D>* tc = DiffTestCaseFactory<D>::Create(args.Problem);
	// f = d*pi^2 * prod sin(pi x_i), u = prod sin(pi x_i), homogeneous Dirichlet.
	if constexpr (D == 2)
	{
		tc->SourceFunction = [](const DomPoint& p) { return 2 * M_PI * M_PI * sin(M_PI * p.X) * sin(M_PI * p.Y); };
		tc->ExactSolution = [](const DomPoint& p) { return sin(M_PI * p.X) * sin(M_PI * p.Y); };
	}
	else
	{
		tc->SourceFunction = [](const DomPoint& p) { return 3 * M_PI * M_PI * sin(M_PI * p.X) * sin(M_PI * p.Y) * sin(M_PI * p.Z); };
		tc->ExactSolution = [](const DomPoint& p) { return sin(M_PI * p.X) * sin(M_PI * p.Y) * sin(M_PI * p.Z); };
	}

	Mesh<D>* mesh;
	if constexpr (D == 2)
		mesh = new Square_TriangularMesh(n, n);
	else
		mesh = new Cube_CartesianTetrahedralMesh(n);
	mesh->SetDiffusionField(&tc->DiffField);
	mesh->SetBoundaryConditions(&tc->BC);

	auto* rb = FunctionalBasisFactory<D>::Create(args.Discretization.ElemBasisCode, k + 1, false);
	auto* cb = FunctionalBasisFactory<D>::Create(args.Discretization.ElemBasisCode, k, false);
	auto* fb = FunctionalBasisFactory<D - 1>::Create(args.Discretization.FaceBasisCode, k, false);
	auto* hho = new HHOParameters<D>(mesh, "hho", rb, cb, fb, args.Discretization.OrthogonalizeElemBasesCode, args.Discretization.OrthogonalizeFaceBasesCode);
	auto* pb = new Diffusion_HHO<D>(mesh, tc, hho, true, false);
	pb->Assemble(args.Actions, ExportModule(""));

	// Fine-level face geometry (face Number -> vertices in the face's own order).
	{
		int nf = (int)pb->HHO->nInteriorAndNeumannFaces;
		std::vector<double> geo((size_t)nf * D * D, 0.0);
		for (Face<D>* f : mesh->Faces)
		{
			if (f->HasDirichletBC()) continue;
			auto vs = f->Vertices();
			for (int v = 0; v < D && v < (int)vs.size(); v++)
			{
				geo[((size_t)f->Number * D + v) * D + 0] = vs[v]->X;
				if (D > 1) geo[((size_t)f->Number * D + v) * D + 1] = vs[v]->Y;
				if (D > 2) geo[((size_t)f->Number * D + v) * D + 2] = vs[v]->Z;
			}
		}
		WriteArray(outdir + "/L0_face_vertices.f64", geo.data(), geo.size());
	}

	int bs = fb->Size();
	Solver* s = SolverFactory<D>::CreateSolver(args, pb, bs, ExportModule(""));
	FlexibleConjugateGradient* fcg = dynamic_cast<FlexibleConjugateGradient*>(s);
	if (!fcg) { fprintf(stderr, "unexpected solver type\n"); return 3; }
	Timer setupTimer; setupTimer.Start();
	fcg->Setup(pb->A);
	setupTimer.Stop();

	Multigrid* mg = dynamic_cast<Multigrid*>(PrecondSolver(fcg->Precond));
	if (!mg) { fprintf(stderr, "unexpected preconditioner type\n"); return 3; }
	int nLevels = 0;
	std::vector<int> blockSizes;
	Level* last = nullptr;
	for (Level* l = MGFine(mg); l; l = l->CoarserLevel, nLevels++)
	{
		std::string p = outdir + "/L" + std::to_string(l->Number);
		DumpCSR(p + "_A", *l->OperatorMatrix);
		if (!l->IsCoarsestLevel())
			DumpCSR(p + "_P", LevelP(l));
		blockSizes.push_back(l->BlockSizeForBlockSmoothers());
		last = l;
	}
	const int pLevels = nLevels;
	// p-multigrid with an h-multigrid coarse solver: its levels below its finest (which is the
	// lowest-degree p-level), numbered on.
	if (Multigrid* inner = precond == "p_mg" ? dynamic_cast<Multigrid*>(mg->CoarseSolver) : nullptr)
	{
		Level* f = MGFine(inner);
		if (f && !f->IsCoarsestLevel())
			DumpCSR(outdir + "/L" + std::to_string(last->Number) + "_P", LevelP(f));
		int number = last->Number;
		for (Level* l = f ? f->CoarserLevel : nullptr; l; l = l->CoarserLevel, nLevels++)
		{
			std::string p = outdir + "/L" + std::to_string(++number);
			DumpCSR(p + "_A", *l->OperatorMatrix);
			if (!l->IsCoarsestLevel())
				DumpCSR(p + "_P", LevelP(l));
			blockSizes.push_back(l->BlockSizeForBlockSmoothers());
		}
	}
	WriteArray(outdir + "/b.f64", pb->b.data(), (size_t)pb->b.rows());
	WriteArray(outdir + "/block_sizes.i32", blockSizes.data(), blockSizes.size());

	std::ostringstream meta;
	meta << "{\"dim\": " << D << ", \"n\": " << n << ", \"k\": " << k << ", \"block_size\": " << bs
	     << ", \"levels\": " << nLevels << ", \"p_levels\": " << pLevels << ", \"pre\": \"" << pre
	     << "\", \"post\": \"" << post << "\", \"precond\": \"" << precond << "\", \"coarse_solver\": \""
	     << coarseSolver << "\", \"setup_s\": " << setupTimer.Elapsed().InSeconds();

	if (solve)
	{
		std::vector<double> hist;
		fcg->OnIterationEnd = [&hist](const IterationResult& r) { hist.push_back(r.NormalizedResidualNorm); };
		Timer t; t.Start();
		Vector x = static_cast<IterativeSolver*>(fcg)->Solve(pb->b, std::string("0"));
		t.Stop();
		WriteArray(outdir + "/x.f64", x.data(), (size_t)x.rows());
		WriteArray(outdir + "/history.f64", hist.data(), hist.size());
		meta << ", \"iterations\": " << fcg->IterationCount << ", \"solve_s\": " << t.Elapsed().InSeconds();
		// Post-processing as Program_Diffusion_HHO::Execute (src/Program/Program_Diffusion_HHO.h:319-390):
		// cell unknowns, k+1 reconstruction, relative L2 error against the exact solution.
		Vector recon = pb->ReconstructHigherOrderApproximationFromFaceCoeffs(x);
		double l2 = pb->L2Error(tc->ExactSolution, recon);
		meta.precision(17);
		meta << ", \"l2_error\": " << l2;
	}
	meta << "}\n";
	WriteText(outdir + "/meta.json", meta.str());
	return 0;
}

// ---------------------------------------------------------------------------
// solve: the reference multigrid classes on a given algebraic hierarchy.
class AlgebraicLevel : public Level
{
public:
	SparseMatrix A_;
	SparseMatrix P_;
	int blockSize = 1;
	bool hasP = false;

	AlgebraicLevel(int number) : Level(number) {}
	int PolynomialDegree() override { return 1; }
	int BlockSizeForBlockSmoothers() override { return blockSize; }
	BigNumber NUnknowns() override { return A_.rows(); }
	void CoarsenMesh(H_CoarsStgy, FaceCoarseningStrategy, FaceCollapsing, double, bool& noCoarser, bool& coarsest) override
	{
		noCoarser = false;
		coarsest = false;
	}
protected:
	void SetupDiscretizedOperator() override { this->OperatorMatrix = &A_; }
	void SetupProlongation() override { this->P = P_; }
	// Same as LevelForHHO::SetupRestriction with RestrictionScalingFactor() == 1.
	void SetupRestriction() override { this->R = this->P.transpose().eval(); }
};

class AlgebraicMultigrid : public Multigrid
{
public:
	std::vector<AlgebraicLevel*> levels;
	AlgebraicMultigrid(int nLevels) : Multigrid(nLevels) {}
	void Serialize(ostream& os) const override { os << "AlgebraicMultigrid"; }
protected:
	Level* CreateFineLevel() const override { return levels[0]; }
	Level* CreateCoarseLevel(Level* fineLevel, CoarseningType, int) override { return levels[fineLevel->Number + 1]; }
};

static int RunSolve(const std::string& dir, const std::string& pre, const std::string& post, const std::string& krylov, double tol, int maxit, char cycle, double omega)
{
	auto meta = ReadArray<int>(dir + "/levels.i32"); // [nLevels, blockSize]
	int nLevels = meta[0], bs = meta[1];
	Utils::ProgramArgs = ProgramArguments();

	AlgebraicMultigrid* mg = new AlgebraicMultigrid(nLevels);
	for (int l = 0; l < nLevels; l++)
	{
		auto* lev = new AlgebraicLevel(l);
		lev->blockSize = bs;
		lev->A_ = LoadCSR(dir + "/L" + std::to_string(l) + "_A");
		if (l < nLevels - 1)
			lev->P_ = LoadCSR(dir + "/L" + std::to_string(l) + "_P");
		mg->levels.push_back(lev);
	}
	// Parameters as SolverFactory::SetMultigridParameters (src/Solver/SolverFactory.h:236-310).
	// "-cycle V,1,1" / "-cycle W,1,1" (src/main.cpp:1179-1215)
	mg->Cycle = cycle;
	mg->WLoops = cycle == 'W' ? 2 : 1;
	mg->PreSmootherCode = pre;
	mg->PostSmootherCode = post;
	mg->PreSmoothingIterations = 1;
	mg->PostSmoothingIterations = 1;
	mg->BlockSizeForBlockSmoothers = bs;
	// "-w": Multigrid::RelaxationParameter (bj, and block SOR for the GS codes when != 1)
	mg->RelaxationParameter = omega;
	mg->H_CS = H_CoarsStgy::StandardCoarsening;
	mg->CoarseSolver = new EigenSparseCholesky();

	const SparseMatrix& A0 = mg->levels[0]->A_;
	auto bvec = ReadArray<double>(dir + "/b.f64");
	Vector b = Eigen::Map<Vector>(bvec.data(), (Eigen::Index)bvec.size());

	IterativeSolver* it = nullptr;
	FlexibleConjugateGradient* fcg = nullptr;
	ConjugateGradient* cg = nullptr;
	if (krylov == "cg")
	{
		cg = new ConjugateGradient();
		cg->Precond = SolverPreconditioner(mg);
		it = cg;
	}
	else
	{
		fcg = new FlexibleConjugateGradient(1);
		fcg->Precond = SolverPreconditioner(mg);
		it = fcg;
	}
	it->Tolerance = tol;
	it->MaxIterations = maxit;
	it->PrintIterationResults = false;
	it->Setup(A0);

	std::vector<double> hist;
	it->OnIterationEnd = [&hist](const IterationResult& r) { hist.push_back(r.NormalizedResidualNorm); };
	Timer t; t.Start();
	Vector x = it->Solve(b, std::string("0"));
	t.Stop();
	WriteArray(dir + "/out_x.f64", x.data(), (size_t)x.rows());
	WriteArray(dir + "/out_history.f64", hist.data(), hist.size());
	std::ostringstream meta2;
	meta2 << "{\"iterations\": " << it->IterationCount << ", \"solve_s\": " << t.Elapsed().InSeconds() << "}\n";
	WriteText(dir + "/out_meta.json", meta2.str());
	return 0;
}

int main(int argc, char** argv)
{
	if (argc < 2) { fprintf(stderr, "usage: ref_driver gen|solve ...\n"); return 1; }
	std::string mode = argv[1];
	std::string pre = "bgs", post = "rbgs", krylov = "fcg";
	char cycle = 'V';
	double tol = 1e-8, omega = 1.0;
	int maxit = 200;
	bool solve = true;
	std::string coarseSolver = "ch";
	P_CoarsStgy pcs = P_CoarsStgy::Minus2;
	std::vector<std::string> pos;
	for (int i = 2; i < argc; i++)
	{
		std::string a = argv[i];
		if (a == "--smoothers" && i + 1 < argc) ParseSmoothers(argv[++i], pre, post);
		else if (a == "--krylov" && i + 1 < argc) krylov = argv[++i];
		else if (a == "--tol" && i + 1 < argc) tol = atof(argv[++i]);
		else if (a == "--omega" && i + 1 < argc) omega = atof(argv[++i]);
		else if (a == "--maxit" && i + 1 < argc) maxit = atoi(argv[++i]);
		else if (a == "--no-solve") solve = false;
		else if (a == "--cycle" && i + 1 < argc) cycle = argv[++i][0];
		else if (a == "--coarse-solver" && i + 1 < argc) coarseSolver = argv[++i];
		else if (a == "--p-cs" && i + 1 < argc) pcs = std::string(argv[++i]) == "minus1" ? P_CoarsStgy::Minus1 : P_CoarsStgy::Minus2;
		else pos.push_back(a);
	}
	std::cout.setstate(std::ios_base::failbit); // the reference logs to stdout; keep it quiet
	int rc = 1;
	if (mode == "gen" && pos.size() == 4)
	{
		int dim = atoi(pos[0].c_str()), n = atoi(pos[1].c_str()), k = atoi(pos[2].c_str());
		if (dim == 2) rc = RunGen<2>(n, k, pos[3], pre, post, solve);
		else rc = RunGen<3>(n, k, pos[3], pre, post, solve);
	}
	else if (mode == "genp" && pos.size() == 4)
	{
		int dim = atoi(pos[0].c_str()), n = atoi(pos[1].c_str()), k = atoi(pos[2].c_str());
		if (dim == 2) rc = RunGen<2>(n, k, pos[3], pre, post, solve, "p_mg", coarseSolver, pcs);
		else rc = RunGen<3>(n, k, pos[3], pre, post, solve, "p_mg", coarseSolver, pcs);
	}
	else if (mode == "solve" && pos.size() == 1)
		rc = RunSolve(pos[0], pre, post, krylov, tol, maxit, cycle, omega);
	else
		fprintf(stderr, "bad arguments\n");
	std::cout.clear();
	return rc;
}
