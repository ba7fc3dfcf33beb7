// Replacement for the reference's src/LinearSystem.cpp in the oracle build.
// The reference hands the assembled block system to PARDISO / FASP / PETSc /
// SAMG, none of which is available here; this translation unit keeps the
// LinearSystem interface (include/LinearSystem.hpp) and plugs in a dense LU
// solve (LAPACK dgesv) of the block-CSR matrix, adequate for the few thousand
// unknowns of the fixture decks.  Harness code, not part of the product.
#include "LinearSystem.hpp"
#include "DenseMat.hpp"

namespace {

class DenseLUSolver : public LinearSolver
{
public:
    explicit DenseLUSolver(OCPMatrix& m) : mat(m) {}

    void AssembleMat(OCPMatrix& m, const Domain*) override
    {
        const OCP_USI nb  = m.nb;
        const OCP_USI dim = m.dim;
        n = dim * nb;
        // column-major dense copy for dgesv
        A.assign(static_cast<size_t>(n) * n, 0.0);
        for (OCP_USI r = 0; r < dim; r++) {
            const auto& cols = m.colId[r];
            const auto& vals = m.val[r];
            for (size_t k = 0; k < cols.size(); k++) {
                const OCP_USI c = cols[k];
                for (OCP_USI i = 0; i < nb; i++)
                    for (OCP_USI j = 0; j < nb; j++)
                        A[static_cast<size_t>(c * nb + j) * n + (r * nb + i)] +=
                            vals[k * nb * nb + i * nb + j];
            }
        }
        rhs.assign(m.b.begin(), m.b.begin() + n);
    }

    OCP_INT Solve() override
    {
        std::vector<INT> piv(n);
        INT nrhs = 1, info = 0, N = static_cast<INT>(n);
        dgesv_(&N, &nrhs, A.data(), &N, piv.data(), rhs.data(), &N, &info);
        if (info != 0) return -1;
        std::copy(rhs.begin(), rhs.end(), mat.u.begin());
        return 1;
    }

    USI GetNumIters() const override { return 1; }

private:
    OCPMatrix&           mat;
    OCP_USI              n{0};
    std::vector<OCP_DBL> A;
    std::vector<OCP_DBL> rhs;
};

} // namespace

USI LinearSystem::Setup(const OCPModel& model, const string& dir, const string& file,
                        const Domain& d, const USI& nb)
{
    solveDir = dir;
    domain   = &d;
    nbs.push_back(nb);
    mat.Allocate(*domain, nb);
    SetupLinearSolver(model, file);
    return LS.size() - 1;
}

void LinearSystem::SetWorkLS(const USI& i)
{
    wIndex = i;
    mat.SetBlockDim(nbs[wIndex]);
}

void LinearSystem::SetupLinearSolver(const OCPModel&, const string&)
{
    LS.push_back(new DenseLUSolver(mat));
    LStype.push_back(OCPLStype::none);
}

void LinearSystem::AssembleMatLinearSolver() { LS[wIndex]->AssembleMat(mat, domain); }

OCP_INT LinearSystem::Solve() { return LS[wIndex]->Solve(); }
