// Compile-and-link check of include/fhg_reference_adapter.hpp against the reference headers
// (no GPU needed: the program is built, not run, in environments without one). With a GPU it
// solves the reference's 2D config-1 problem through the adapter and prints the iterations.
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

int main()
{
    ProgramArguments args;
    args.Problem.Dimension = 2;
    args.Problem.GeoCode = args.Problem.TestCaseCode = "square";
    args.Problem.BCCode = "d";
    args.Solver.MG.H_CS = H_CoarsStgy::StandardCoarsening;
    args.Solver.MG.GMG_H_Prolong = GMG_H_Prolongation::CellInterp_Trace;
    args.Actions.LogAssembly = false;
    Utils::ProgramArgs = args;
    GaussLegendre::Init();
    auto* tc = DiffTestCaseFactory<2>::Create(args.Problem);
    Mesh<2>* mesh = new Square_TriangularMesh(32, 32);
    mesh->SetDiffusionField(&tc->DiffField);
    mesh->SetBoundaryConditions(&tc->BC);
    auto* rb = FunctionalBasisFactory<2>::Create("monomials", 2, false);
    auto* cb = FunctionalBasisFactory<2>::Create("monomials", 1, false);
    auto* fb = FunctionalBasisFactory<1>::Create("legendre", 1, false);
    auto* hho = new HHOParameters<2>(mesh, "hho", rb, cb, fb, 1, 0);
    auto* pb = new Diffusion_HHO<2>(mesh, tc, hho, true, false);
    pb->Assemble(args.Actions, ExportModule(""));
    GpuFcgMg<2> solver(pb, args, fb->Size());
    solver.Tolerance = 1e-8;
    solver.Setup(pb->A);
    Vector x = solver.Solve(pb->b, "0");
    std::cerr << "iterations " << solver.IterationCount << std::endl;
    return 0;
}
