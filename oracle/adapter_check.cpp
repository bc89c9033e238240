// Compile-and-link check of include/fhg_reference_adapter.hpp against the reference headers
// (TEST INFRASTRUCTURE). `adapter_check --map` needs no GPU: it prints the fhg_options the adapter
// derives from several ProgramArguments settings. `adapter_check --levels <dim> <n> <k> <solver>
// <coarse solver>` needs no GPU either: it builds the reference's problem and the adapter's host
// hierarchy and prints every level (rows, block size, prolongation shape) on stderr. Without arguments (GPU
// needed) it solves the reference's 2D problem on a 32 x 32 triangle mesh (k = 1) through the
// adapter and prints the iterations.
#include "ProgramArguments.h"
#include "Discretizations/DG/Diffusion_DG.h"
#include "TestCases/Diffusion/DiffTestCaseFactory.h"
#include "Mesher/InHouse/Square_CartesianMesh.h"
#include "Mesher/InHouse/Square_TriangularMesh.h"
#include "Mesher/InHouse/Cube_CartesianTetrahedralMesh.h"
#include "FunctionalBasis/FunctionalBasisFactory.h"
#include "Discretizations/HHO/Diffusion_HHO.h"
#include "Solver/SolverFactory.h"
#include "fhg_reference_adapter.hpp"

static void print_options(const char* name, const ProgramArguments& a)
{
    const fhg_options o = GpuFcgMg<2>::MapArguments(a);
    std::cout << name << " krylov=" << o.krylov << " pre=" << o.pre_smoother << " post=" << o.post_smoother
              << " npre=" << o.pre_iterations << " npost=" << o.post_iterations << " omega=" << o.omega
              << " w_loops=" << o.w_loops << " galerkin=" << o.galerkin << " tol=" << o.tolerance
              << " maxit=" << o.max_iterations << " cpre=" << o.coarse_pre_iterations
              << " cpost=" << o.coarse_post_iterations << std::endl;
}

static int map_check()
{
    ProgramArguments a;
    a.Solver.SolverCode = "fcgmg";
    print_options("default", a);
    a.Solver.MG.PostSmootherCode = "<symmetric smoother>";
    a.Solver.MG.PreSmootherCode = "abgs";
    a.Solver.MG.PreSmoothingIterations = 3;
    print_options("abgs3_symmetric", a);
    a.Solver.MG.PreSmootherCode = "hbgs";
    print_options("hbgs_symmetric", a);
    ProgramArguments w;
    w.Solver.SolverCode = "cg";
    w.Solver.PreconditionerCode = "mg";
    w.Solver.MG.CycleLetter = 'W';
    w.Solver.MG.WLoops = 2;
    w.Solver.MG.UseGalerkinOperator = true;
    w.Solver.MG.PreSmootherCode = "bsor";
    w.Solver.MG.PostSmootherCode = "rbsor";
    w.Solver.RelaxationParameter = 1.2;
    w.Solver.Tolerance = 1e-10;
    w.Solver.MaxIterations = 50;
    print_options("cg_w_sor", w);
    ProgramArguments k;
    k.Solver.SolverCode = "cgmg";
    k.Solver.MG.CycleLetter = 'K';
    k.Solver.MG.PreSmootherCode = "bj23";
    k.Solver.MG.PostSmootherCode = "<symmetric smoother>";
    print_options("cgmg_k_bj23", k);
    ProgramArguments p;
    p.Solver.SolverCode = "fcgp_mg";
    print_options("fcgp_mg", p);
    ProgramArguments q;
    q.Solver.SolverCode = "cg";
    q.Solver.PreconditionerCode = "p_mg";
    q.Solver.MG.CoarseSolverCode = "mg";
    print_options("cg_p_mg_cs_mg", q);
    return 0;
}

// The reference's problem (Dirichlet, the built-in test case) on the in-house triangle or
// tetrahedral mesh with the default bases of main.cpp:1703-1735, assembled.
template <int D>
static Diffusion_HHO<D>* make_problem(ProgramArguments& args, int n, int k)
{
    args.Problem.Dimension = D;
    args.Problem.GeoCode = args.Problem.TestCaseCode = D == 2 ? "square" : "cube";
    args.Problem.BCCode = "d";
    args.Solver.MG.H_CS = H_CoarsStgy::StandardCoarsening;
    args.Solver.MG.GMG_H_Prolong = GMG_H_Prolongation::CellInterp_Trace;
    args.Actions.LogAssembly = false;
    Utils::ProgramArgs = args;
    GaussLegendre::Init();
    auto* tc = DiffTestCaseFactory<D>::Create(args.Problem);
    Mesh<D>* mesh;
    if constexpr (D == 2)
        mesh = new Square_TriangularMesh(n, n);
    else
        mesh = new Cube_CartesianTetrahedralMesh(n);
    mesh->SetDiffusionField(&tc->DiffField);
    mesh->SetBoundaryConditions(&tc->BC);
    auto* rb = FunctionalBasisFactory<D>::Create("monomials", k + 1, false);
    auto* cb = FunctionalBasisFactory<D>::Create("monomials", k, false);
    auto* fb = FunctionalBasisFactory<D - 1>::Create(D == 2 ? "legendre" : "monomials", k, false);
    auto* hho = new HHOParameters<D>(mesh, "hho", rb, cb, fb, 1, D == 2 ? 0 : 1);
    auto* pb = new Diffusion_HHO<D>(mesh, tc, hho, true, false);
    pb->Assemble(args.Actions, ExportModule(""));
    return pb;
}

template <int D>
static int levels_check(int n, int k, const std::string& solver, const std::string& coarse)
{
    ProgramArguments args;
    args.Solver.SolverCode = solver;
    args.Solver.MG.CoarseSolverCode = coarse;
    Diffusion_HHO<D>* pb = make_problem<D>(args, n, k);
    GpuFcgMg<D> s(pb, args, pb->HHO->nFaceUnknowns);
    s.BuildHostHierarchy(pb->A);
    const auto levels = s.Levels();
    // on stderr: the reference logs its setup on stdout
    for (size_t l = 0; l < levels.size(); l++)
        std::cerr << "level" << l << " rows=" << levels[l].A->rows() << " bs=" << levels[l].blockSize
                  << " p_rows=" << (levels[l].P ? levels[l].P->rows() : 0)
                  << " p_cols=" << (levels[l].P ? levels[l].P->cols() : 0) << std::endl;
    return 0;
}

int main(int argc, char** argv)
{
    if (argc > 1 && std::string(argv[1]) == "--map")
        return map_check();
    if (argc > 6 && std::string(argv[1]) == "--levels")
    {
        const int dim = atoi(argv[2]), n = atoi(argv[3]), k = atoi(argv[4]);
        return dim == 2 ? levels_check<2>(n, k, argv[5], argv[6]) : levels_check<3>(n, k, argv[5], argv[6]);
    }
    if (argc > 2 && std::string(argv[1]) == "--reject")
    {   // an unsupported setting: the mapping must end in Utils::FatalError
        ProgramArguments a;
        a.Solver.SolverCode = "fcgmg";
        const std::string what(argv[2]);
        if (what == "solver") a.Solver.SolverCode = "bicgstab";
        if (what == "smoother") a.Solver.MG.PreSmootherCode = "gs";
        if (what == "coarse") a.Solver.MG.CoarseSolverCode = "fcgmg";
        if (what == "variable") a.Solver.MG.CoarseLevelChangeSmoothingCoeff = 1;
        if (what == "coarse_mg") a.Solver.MG.CoarseSolverCode = "mg";   // only under the p-multigrid
        if (what == "p_mg_w")
        {
            a.Solver.SolverCode = "fcgp_mg";
            a.Solver.MG.CoarseSolverCode = "mg";
            a.Solver.MG.CycleLetter = 'W';
        }
        print_options("accepted", a);
        return 0;
    }
    ProgramArguments args;
    args.Solver.SolverCode = "fcgmg";
    Diffusion_HHO<2>* pb = make_problem<2>(args, 32, 1);
    GpuFcgMg<2> solver(pb, args, pb->HHO->nFaceUnknowns);
    solver.Tolerance = 1e-8;
    solver.Setup(pb->A);
    Vector x = solver.Solve(pb->b, "0");
    std::cerr << "iterations " << solver.IterationCount << std::endl;
    return 0;
}
