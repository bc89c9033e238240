// C++ adapter that plugs the GB300 solve phase (include/fhg.h, libfhg.so) into fhhos4's
// solver interface. It is meant to be added to the fhhos4 source tree (for instance as
// src/Solver/Gpu/GpuFcgMg.h) and compiles against the reference headers unmodified:
// protected members are read through pointers-to-member of local helper types.
//
// GpuFcgMg<Dim> is an IterativeSolver (src/Solver/IterativeSolver.h:6-191): Setup(A) runs the
// reference's own MultigridForHHO<Dim>::Setup on the host (src/Solver/Multigrid/Multigrid.h:88-313),
// or P_MultigridForHHO<Dim>'s for the p-multigrid preconditioner (with, for "-cs mg", the
// MultigridForHHO coarse solver of the lowest degree SolverFactory.h:289-309 builds), hands every
// level's operator, block size and prolongation to the GPU and builds the device hierarchy;
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
    Multigrid* _mg = nullptr;  // host-side hierarchy builder (reference code)
    bool _p = false;           // p-multigrid: P_MultigridForHHO, its levels' block sizes differ
    int _device = 0;
    fhg_options _opts;

public:
    // One level of the hierarchy the reference's classes built: operator, prolongation to the next
    // level (null on the coarsest) and block size.
    struct HostLevel
    {
        const SparseMatrix* A;
        const SparseMatrix* P;
        int blockSize;
    };

    GpuFcgMg(Diffusion_HHO<Dim>* problem, const ProgramArguments& args, int blockSize, int device = 0)
    {
        _opts = MapArguments(args);
        const MultigridArguments& m = args.Solver.MG;
        _p = UsesPMultigrid(args.Solver);
        if (_p)
        {
            // SolverFactory.h:201-211 with SetMultigridParameters; the coarse solver of "-cs mg" as
            // SolverFactory.h:289-309 configures it (the other fields at their defaults), its
            // problem set by P_MultigridForHHO::InitializeCoarseSolver
            auto* pmg = new P_MultigridForHHO<Dim>(problem);
            pmg->MatrixMaxSizeForCoarsestLevel = m.MatrixMaxSizeForCoarsestLevel;
            pmg->UseGalerkinOperator = m.UseGalerkinOperator;
            pmg->P_CS = m.P_CS;
            pmg->HP_CS = HP_CoarsStgy::P_only;
            pmg->PreSmoothingIterations = 0;   // smoothers run on the GPU: no host smoother setup needed
            pmg->PostSmoothingIterations = 0;
            if (m.CoarseSolverCode == "mg")
            {
                MultigridArguments c;
                c.GMG_H_Prolong = m.GMG_H_Prolong;
                c.H_CS = m.H_CS;
                c.FaceCoarseningStgy = m.FaceCoarseningStgy;
                auto* inner = new MultigridForHHO<Dim>(0);
                ConfigureH(inner, c);
                pmg->CoarseSolver = inner;
            }
            else
                pmg->CoarseSolver = new EigenSparseCholesky();
            _mg = pmg;
        }
        else
        {
            auto* mg = new MultigridForHHO<Dim>(m.Levels);
            ConfigureH(mg, m);
            mg->InitializeWithProblem(problem);
            mg->BlockSizeForBlockSmoothers = blockSize;
            _mg = mg;
        }
        this->Tolerance = args.Solver.Tolerance;
        this->MaxIterations = args.Solver.MaxIterations;
        _device = device;
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
        BuildHostHierarchy(A);
        _opts.tolerance = this->Tolerance;   // the caller may have changed them after construction
        _opts.max_iterations = this->MaxIterations;
        if (!_ctx)
            Check(fhg_create(&_ctx, _device));
        const std::vector<HostLevel> levels = Levels();
        for (int l = 0; l < (int)levels.size(); l++)
        {
            const HostLevel& L = levels[l];
            Check(fhg_set_level(_ctx, l, L.blockSize, (int)L.A->rows(), L.A->outerIndexPtr(), L.A->innerIndexPtr(),
                                L.A->valuePtr()));
            if (L.P)
                Check(fhg_set_prolongation(_ctx, l, (int)L.P->rows(), (int)L.P->cols(), L.P->outerIndexPtr(),
                                           L.P->innerIndexPtr(), L.P->valuePtr()));
        }
        Check(fhg_setup(_ctx, (int)levels.size(), &_opts));
    }

    // The reference's own multigrid setup on the host (no device call): MultigridForHHO's, or
    // P_MultigridForHHO's with its coarse solver's.
    void BuildHostHierarchy(const SparseMatrix& A) { _mg->Setup(A); }

    // The levels the device hierarchy is made of, after BuildHostHierarchy. For the p-multigrid with
    // the h-multigrid coarse solver, that solver's levels below its finest (the lowest degree, the
    // last p-level) continue the hierarchy, and its one cycle (no pre-smoothing, 3 / 6 post-smoothing
    // steps) runs as the coarse part of the V-cycle.
    std::vector<HostLevel> Levels() const
    {
        std::vector<HostLevel> out;
        Level* fine = _mg->*(&fhg_detail::MultigridFineLevel::_fineLevel);
        for (Level* lev = fine; lev; lev = lev->CoarserLevel)
            out.push_back({lev->OperatorMatrix, lev->IsCoarsestLevel() ? nullptr : &ProlongationOf(lev),
                           _p ? lev->BlockSizeForBlockSmoothers() : _mg->BlockSizeForBlockSmoothers});
        if (Multigrid* inner = _p ? dynamic_cast<Multigrid*>(_mg->CoarseSolver) : nullptr)
        {
            if (out.size() != 2)
                Utils::FatalError("GPU solver: with '-cs mg' the p-multigrid must have exactly two levels (the "
                                  "finest and the lowest degree): other levels would need smoothing counts of their own");
            Level* f = inner->*(&fhg_detail::MultigridFineLevel::_fineLevel);
            const int bs = out.back().blockSize;
            if (f && !f->IsCoarsestLevel())
            {
                out.back().P = &ProlongationOf(f);
                for (Level* lev = f->CoarserLevel; lev; lev = lev->CoarserLevel)
                    out.push_back({lev->OperatorMatrix, lev->IsCoarsestLevel() ? nullptr : &ProlongationOf(lev), bs});
            }
        }
        return out;
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

    static const SparseMatrix& ProlongationOf(Level* lev) { return lev->*(&fhg_detail::LevelProlongation::P); }

    // The h-multigrid fields SolverFactory sets for "-s mg" (SolverFactory.h:183-200, 236-256).
    static void ConfigureH(MultigridForHHO<Dim>* mg, const MultigridArguments& m)
    {
        mg->UseHigherOrderReconstruction = m.UseHigherOrderReconstruction;
        mg->H_Prolongation = m.GMG_H_Prolong;
        mg->UseHeterogeneousWeighting = m.UseHeterogeneousWeighting;
        mg->MatrixMaxSizeForCoarsestLevel = m.MatrixMaxSizeForCoarsestLevel;
        mg->UseGalerkinOperator = m.UseGalerkinOperator;
        mg->H_CS = m.H_CS;
        mg->FaceCoarseningStgy = m.FaceCoarseningStgy;
        mg->BdryFaceCollapsing = m.BoundaryFaceCollapsing;
        mg->NumberOfMeshes = m.NumberOfMeshes;
        mg->CoarseningFactor = m.CoarseningFactor;
        mg->PreSmoothingIterations = 0;   // smoothers run on the GPU: no host smoother setup needed
        mg->PostSmoothingIterations = 0;
        mg->CoarseSolver = new EigenSparseCholesky();
    }

    // "-s fcgp_mg" / "-s cgp_mg" or "-s fcg|cg -p p_mg" (SolverFactory.h:125-181, 201-211)
    static bool UsesPMultigrid(const SolverArguments& s)
    {
        return s.SolverCode == "fcgp_mg" || s.SolverCode == "cgp_mg" ||
               ((s.SolverCode == "fcg" || s.SolverCode == "cg") && s.PreconditionerCode == "p_mg");
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
        const bool pc_mg = s.PreconditionerCode == "mg" || s.PreconditionerCode == "p_mg";
        const bool p = UsesPMultigrid(s);
        if (code == "fcgmg" || code == "fcgp_mg" || (code == "fcg" && pc_mg))
            o.krylov = FHG_KRYLOV_FCG;
        else if (code == "cgmg" || code == "cgp_mg" || (code == "cg" && pc_mg))
            o.krylov = FHG_KRYLOV_CG;
        else
            Utils::FatalError("GPU solver: solver code '" + code + "' (preconditioner '" + s.PreconditionerCode +
                              "') is not supported; use fcgmg, cgmg, fcgp_mg or cgp_mg");
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
        if (p && mg.CoarseSolverCode == "mg")
        {
            // one cycle of the lowest degree's h-multigrid (SolverFactory.h:299-308), V-cycle with no
            // pre-smoothing and 3 (2D) or 6 (3D) post-smoothing steps
            if (mg.CycleLetter != 'V')
                Utils::FatalError("GPU solver: '-cs mg' under the p-multigrid needs a V-cycle");
            o.coarse_pre_iterations = 0;
            o.coarse_post_iterations = Dim == 2 ? 3 : 6;
        }
        else if (mg.CoarseSolverCode != "ch" && mg.CoarseSolverCode != "lu")
            Utils::FatalError("GPU solver: coarse solver '" + mg.CoarseSolverCode +
                              "' is not supported; the coarsest level is solved directly (ch / lu)" +
                              (p ? " or, under the p-multigrid, by one h-multigrid cycle (mg)" : ""));
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
