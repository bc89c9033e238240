// C++ adapter that plugs the GB300 solve phase (include/fhg.h, libfhg.so) into fhhos4's
// solver interface. It is meant to be added to the fhhos4 source tree (for instance as
// src/Solver/Gpu/GpuFcgMg.h) and compiles against the reference headers unmodified:
// protected members are read through pointers-to-member of local helper types.
//
// GpuFcgMg<Dim> is an IterativeSolver (src/Solver/IterativeSolver.h:6-191): Setup(A) runs the
// reference's own MultigridForHHO<Dim>::Setup on the host (src/Solver/Multigrid/Multigrid.h:88-313),
// hands every level's operator and prolongation to the GPU and builds the device hierarchy;
// Solve(b, "0") runs FCG(1) + V-cycle entirely on the GPU (FlexibleConjugateGradient.h:47-171).
// A nonzero status becomes Utils::FatalError (src/Utils/Utils.h:258-264), the reference's
// error convention. No CPU fallback exists for the solve.
#pragma once
#include <string>
#include <vector>

#include "fhg.h"

namespace fhg_detail {
struct LevelProlongation : Level { using Level::P; };
struct MultigridFineLevel : Multigrid { using Multigrid::_fineLevel; };
}  // namespace fhg_detail

template <int Dim>
class GpuFcgMg : public IterativeSolver
{
    fhg_ctx* _ctx = nullptr;
    MultigridForHHO<Dim>* _mg = nullptr;  // host-side hierarchy builder (reference code)
    fhg_options _opts;

public:
    GpuFcgMg(Diffusion_HHO<Dim>* problem, const ProgramArguments& args, int blockSize, int device = 0)
    {
        _opts = MapArguments(args);
        _mg = new MultigridForHHO<Dim>(args.Solver.MG.Levels);
        _mg->UseHigherOrderReconstruction = args.Solver.MG.UseHigherOrderReconstruction;
        _mg->H_Prolongation = args.Solver.MG.GMG_H_Prolong;
        _mg->UseHeterogeneousWeighting = args.Solver.MG.UseHeterogeneousWeighting;
        _mg->InitializeWithProblem(problem);
        _mg->BlockSizeForBlockSmoothers = blockSize;
        _mg->MatrixMaxSizeForCoarsestLevel = args.Solver.MG.MatrixMaxSizeForCoarsestLevel;
        _mg->UseGalerkinOperator = args.Solver.MG.UseGalerkinOperator;
        _mg->H_CS = args.Solver.MG.H_CS;
        _mg->FaceCoarseningStgy = args.Solver.MG.FaceCoarseningStgy;
        _mg->BdryFaceCollapsing = args.Solver.MG.BoundaryFaceCollapsing;
        _mg->NumberOfMeshes = args.Solver.MG.NumberOfMeshes;
        _mg->CoarseningFactor = args.Solver.MG.CoarseningFactor;
        _mg->PreSmoothingIterations = 0;   // smoothers run on the GPU: no host smoother setup needed
        _mg->PostSmoothingIterations = 0;
        _mg->CoarseSolver = new EigenSparseCholesky();
        this->Tolerance = args.Solver.Tolerance;
        this->MaxIterations = args.Solver.MaxIterations;
        Check(fhg_create(&_ctx, device));
    }

    ~GpuFcgMg()
    {
        fhg_destroy(_ctx);
        delete _mg;
    }

    void Serialize(ostream& os) const override { os << "FCG(1) + geometric MG V-cycle on GB300 (libfhg)"; }

    void Setup(const SparseMatrix& A) override
    {
        IterativeSolver::Setup(A);
        _mg->Setup(A);
        _opts.tolerance = this->Tolerance;   // the caller may have changed them after construction
        _opts.max_iterations = this->MaxIterations;
        Level* fine = _mg->*(&fhg_detail::MultigridFineLevel::_fineLevel);
        int l = 0;
        for (Level* lev = fine; lev; lev = lev->CoarserLevel, l++)
        {
            const SparseMatrix& Al = *lev->OperatorMatrix;
            Check(fhg_set_level(_ctx, l, _mg->BlockSizeForBlockSmoothers, (int)Al.rows(), Al.outerIndexPtr(),
                                Al.innerIndexPtr(), Al.valuePtr()));
            if (!lev->IsCoarsestLevel())
            {
                const SparseMatrix& P = lev->*(&fhg_detail::LevelProlongation::P);
                Check(fhg_set_prolongation(_ctx, l, (int)P.rows(), (int)P.cols(), P.outerIndexPtr(),
                                           P.innerIndexPtr(), P.valuePtr()));
            }
        }
        Check(fhg_setup(_ctx, l, &_opts));
    }

    Vector Solve(const Vector& b, string initialGuessCode) override
    {
        if (initialGuessCode.compare("0") != 0)
            Utils::FatalError("the GPU solver starts from x = 0 (initial guess code \"0\")");
        Vector x(b.rows());
        std::vector<double> hist(this->MaxIterations + 1);
        fhg_solve_info info;
        const int rc = fhg_solve(_ctx, b.data(), x.data(), hist.data(), &info);
        this->IterationCount = info.iterations;
        if (this->OnIterationEnd)
        {
            IterationResult r;
            for (int k = 0; k <= info.iterations; k++)
            {
                r.IterationNumber = k;
                r.NormalizedResidualNorm = hist[k];
                this->OnIterationEnd(r);
            }
        }
        Check(rc);
        return x;
    }

private:
    void Check(int rc)
    {
        if (rc != FHG_OK)
            Utils::FatalError(std::string("GPU solver: ") + fhg_last_error(_ctx));
    }

    // The solver arguments the reference's SolverFactory reads for "-s fcgmg" / "-s cgmg"
    // (SolverFactory.h:125-200, SetMultigridParameters SolverFactory.h:236-310), mapped to
    // fhg_options; an argument the GPU path does not implement is an error, never ignored.
public:
    static fhg_options MapArguments(const ProgramArguments& args)
    {
        fhg_options o;
        fhg_default_options(&o);
        const SolverArguments& s = args.Solver;
        const string& code = s.SolverCode;
        const bool pc_mg = s.PreconditionerCode == "mg";
        if (code == "fcgmg" || (code == "fcg" && pc_mg))
            o.krylov = FHG_KRYLOV_FCG;
        else if (code == "cgmg" || (code == "cg" && pc_mg))
            o.krylov = FHG_KRYLOV_CG;
        else
            Utils::FatalError("GPU solver: solver code '" + code + "' (preconditioner '" + s.PreconditionerCode +
                              "') is not supported; use fcgmg or cgmg");
        if (s.StoppingCrit != StoppingCriteria::NormalizedResidual)
            Utils::FatalError("GPU solver: only the normalized-residual stopping criterion is supported");
        if (s.InitialGuessCode != "0")
            Utils::FatalError("GPU solver: the initial guess must be \"0\"");
        const MultigridArguments& mg = s.MG;
        if (mg.CycleLetter == 'V')
            o.w_loops = 1;
        else if (mg.CycleLetter == 'W')
            o.w_loops = mg.WLoops > 1 ? mg.WLoops : 2;
        else if (mg.CycleLetter == 'K')
            o.w_loops = FHG_CYCLE_K;
        else
            Utils::FatalError(std::string("GPU solver: multigrid cycle '") + mg.CycleLetter + "' is not supported");
        if (mg.CoarseLevelChangeSmoothingCoeff != 0)
            Utils::FatalError("GPU solver: level-dependent smoothing steps (-cycle V,a,b,+c) are not supported");
        if (mg.CoarseSolverCode != "ch" && mg.CoarseSolverCode != "lu")
            Utils::FatalError("GPU solver: coarse solver '" + mg.CoarseSolverCode +
                              "' is not supported; the coarsest level is solved directly (ch / lu)");
        o.galerkin = mg.UseGalerkinOperator ? 1 : 0;
        o.pre_iterations = mg.PreSmoothingIterations;
        o.post_iterations = mg.PostSmoothingIterations;
        o.omega = s.RelaxationParameter;
        o.tolerance = s.Tolerance;
        o.max_iterations = s.MaxIterations;
        o.pre_smoother = SmootherCode(mg.PreSmootherCode);
        o.post_smoother = SmootherCode(PostSmootherName(mg));
        return o;
    }

private:

    // "<symmetric smoother>" resolved as SetMultigridParameters does (SolverFactory.h:258-283)
    static string PostSmootherName(const MultigridArguments& mg)
    {
        const string& pre = mg.PreSmootherCode;
        if (mg.PostSmootherCode != "<symmetric smoother>")
            return mg.PostSmootherCode;
        if (pre == "bj23" || pre == "bj" || pre == "sbgs")
            return pre;
        if (pre == "bgs")
            return "rbgs";
        if (pre == "hbgs")
            return "hrbgs";
        if (pre == "abgs" || pre == "asor")
            return mg.PreSmoothingIterations % 2 == 0 ? pre : "r" + pre;
        Utils::FatalError("GPU solver: no symmetric post-smoother for '" + pre + "'");
        return pre;
    }

    // Block smoother codes of SmootherFactory::Create (SmootherFactory.h:37-100). The "hbgs" family
    // maps to the multicolour sweeps; with RelaxationParameter != 1 the GS codes become block SOR.
    static int SmootherCode(const string& c)
    {
        if (c == "bgs" || c == "bsor" || c == "hbgs") return FHG_SMOOTHER_BGS;
        if (c == "rbgs" || c == "rbsor" || c == "hrbgs") return FHG_SMOOTHER_RBGS;
        if (c == "sbgs" || c == "sbsor") return FHG_SMOOTHER_SBGS;
        if (c == "abgs" || c == "absor") return FHG_SMOOTHER_ABGS;
        if (c == "rabgs" || c == "rabsor") return FHG_SMOOTHER_RABGS;
        if (c == "bj") return FHG_SMOOTHER_BJ;
        if (c == "bj23") return FHG_SMOOTHER_BJ23;
        Utils::FatalError("GPU solver: smoother '" + c + "' is not supported (block smoothers only)");
        return -1;
    }
};
