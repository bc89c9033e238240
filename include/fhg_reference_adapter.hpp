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
        _mg = new MultigridForHHO<Dim>(problem, args.Solver.MG.Levels);
        _mg->BlockSizeForBlockSmoothers = blockSize;
        _mg->MatrixMaxSizeForCoarsestLevel = args.Solver.MG.MatrixMaxSizeForCoarsestLevel;
        _mg->H_CS = args.Solver.MG.H_CS;
        _mg->H_Prolongation = args.Solver.MG.GMG_H_Prolong;
        _mg->PreSmoothingIterations = 0;   // smoothers run on the GPU: no host smoother setup needed
        _mg->PostSmoothingIterations = 0;
        _mg->CoarseSolver = new EigenSparseCholesky();
        fhg_default_options(&_opts);
        _opts.pre_iterations = args.Solver.MG.PreSmoothingIterations;
        _opts.post_iterations = args.Solver.MG.PostSmoothingIterations;
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
        _opts.tolerance = this->Tolerance;
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
};
