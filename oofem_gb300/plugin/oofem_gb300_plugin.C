// OOFEM-side binding of liboofem_gb300: a SparseMtrx, a SparseLinearSystemNM and
// GPU-backed element classes, registered through OOFEM's own class-factory
// macros so that an unchanged input file selects the GPU path with
//     smtype 11 lstype 9
// in the LinearStatic / NonLinearStatic (NRSolver) analysis record.
//
// Build this file together with an OOFEM build (it includes the reference's
// headers and links liboofem and liboofem_gb300); load it after liboofem so its
// registrations are the ones in force (link it into the oofem executable with
// --no-as-needed, or LD_PRELOAD it).
//
// Interfaces mirrored:
//   SparseMtrx            src/core/sparsemtrx.h:62-303
//   SparseLinearSystemNM  src/core/sparselinsystemnm.h:58-96
//   IMLSolver keys        src/core/iml/imlsolver.C:66-98 (lstol, lsiter)
//   class factory         src/core/classfactory.h:131,135,149-150
#include "sparsemtrx.h"
#include "sparselinsystemnm.h"
#include "classfactory.h"
#include "engngm.h"
#include "domain.h"
#include "element.h"
#include "dofmanager.h"
#include "dof.h"
#include "node.h"
#include "floatarray.h"
#include "floatmatrix.h"
#include "intarray.h"
#include "timestep.h"
#include "unknownnumberingscheme.h"
#include "convergedreason.h"
#include "inputrecord.h"
#include "error.h"
#include "crosssection.h"
#include "sm/Elements/3D/lspace.h"
#include "sm/Elements/3D/ltrspace.h"
#include "sm/Elements/PlaneStress/planstrss.h"
#include "sm/Materials/isolinearelasticmaterial.h"

#include <cstdlib>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "oofem_gb300.h"

namespace oofem {

#define SMT_GpuCsr ((SparseMtrxType)11)
#define ST_GpuPcg ((LinSystSolverType)9)
#define _IFT_GpuPcgSolver_lstol "lstol"
#define _IFT_GpuPcgSolver_lsiter "lsiter"
#define _IFT_GpuPcgSolver_gpuprec "gpuprec"
#define _IFT_GpuPcgSolver_lsprecond "lsprecond"

static ogb_ctx *gb300_context()
{
    static ogb_ctx *ctx = nullptr;
    if ( !ctx ) {
        const char *dev = std::getenv("OOFEM_GB300_DEVICE");
        if ( ogb_ctx_create(dev ? std::atoi(dev) : 0, & ctx) != OGB_OK ) {
            OOFEM_ERROR("liboofem_gb300: %s", ogb_last_error() );
        }
    }
    return ctx;
}

static void gb300_check(int code, const char *what)
{
    if ( code != OGB_OK ) {
        OOFEM_ERROR("%s: %s", what, ogb_last_error() );
    }
}

class GpuCsrMtrx;
// The GpuCsrMtrx whose element loop is in progress and whose elements are
// evaluated on the device, or null. Only inside that window do the GPU element
// classes hand an empty stiffness to the host loop (EngngModel::assemble skips
// it, engngm.C:913-915); every other caller of the element stiffness -- the
// extrapolated-force loops of the IG_Tangent initial guess
// (EngngModel::assemblePrescribedExtrapolatedForces / assembleExtrapolatedForces,
// engngm.C:1536-1666), other matrices, output -- gets the real matrix. The window
// opens where the drivers start an assembly of this matrix (zero() before
// NonLinearStatic / StaticStructural re-assemble it, nlinearstatic.C:621-641,
// staticstructural.C:418-437; buildInternalStructure() under LinearStatic, which
// assembles right after it, linearstatic.C:197-199) and closes in assembleEnd()
// (engngm.C:1035-1036) or when the matrix is destroyed.
static const GpuCsrMtrx *g_device_assembly = nullptr;

/// SparseMtrx whose storage lives on the GPU: the full-pattern CSR (== CompCol),
/// plus the node-block copy used by the solver when built from a mesh.
class GpuCsrMtrx : public SparseMtrx
{
protected:
    ogb_mtrx *m = nullptr;
    ogb_model *model = nullptr;
    EngngModel *emodel = nullptr;   // model and domain the device elements mirror
    int domainIndex = 1;
    // writes through at(i,j) are kept on the host and flushed before any device use
    mutable std::map< std::pair< int, int >, double >pending;

    void flush() const
    {
        for ( auto &kv : pending ) {
            gb300_check(ogb_mtrx_set_at(m, kv.first.first, kv.first.second, kv.second), "GpuCsrMtrx::at");
        }
        pending.clear();
    }

    // Equation numbers of the device model against OOFEM's own (default numbering,
    // EngngModel::forceEquationNumbering engngm.C:469-530): the same count, and for
    // every node the same DOFs (D_u, D_v[, D_w], master DOFs only) with the same
    // number (free > 0, prescribed 0). Any difference -- renumber 1 (Sloan), slave
    // or extra DOFs, a boundary condition whose activity changed -- means the
    // device pattern and OOFEM's vectors would not line up.
    bool numberingMatches(EngngModel *eModel, int di) const
    {
        if ( !model ) {
            return false;
        }
        Domain *d = eModel->giveDomain(di);
        EModelDefaultEquationNumbering dn;
        int neq = 0, npeq = 0;
        if ( ogb_model_neq(model, & neq, & npeq) != OGB_OK || neq != eModel->giveNumberOfDomainEquations(di, dn) ) {
            return false;
        }
        const int nn = d->giveNumberOfDofManagers();
        const int ndofpn = ( int ) ( eqCache.size() / ( nn > 0 ? nn : 1 ) );
        if ( ( size_t ) nn * ndofpn != eqCache.size() ) {
            return false;
        }
        for ( int i = 1; i <= nn; i++ ) {
            DofManager *dm = d->giveDofManager(i);
            if ( dm->giveNumberOfDofs() != ndofpn ) {
                return false;
            }
            int k = 0;
            for ( Dof *dof : *dm ) {
                if ( !dof->isPrimaryDof() || ( int ) dof->giveDofID() != k + 1 ) {
                    return false;
                }
                const int mine = eqCache [ ( size_t ) ( i - 1 ) * ndofpn + k ];
                if ( dof->giveEquationNumber(dn) != ( mine > 0 ? mine : 0 ) ) {
                    return false;
                }
                k++;
            }
        }
        return true;
    }
    std::vector< int >eqCache;   // device equation numbers (nnodes x ndofpn, +free / -prescribed)

    void dropDeviceElements()
    {
        if ( g_device_assembly == this ) {
            g_device_assembly = nullptr;
        }
        if ( model ) {
            ogb_model_destroy(model);
            model = nullptr;
        }
        eqCache.clear();
    }

    // Mesh of LSpace / LTRSpace / PlaneStress2d elements with isotropic linear
    // elastic materials whose numbering the device reproduces: build the device
    // element backend (K1 + gather assembly). False (host element loop and
    // location arrays) for anything else.
    bool tryDeviceElements(EngngModel *eModel, int di)
    {
        Domain *d = eModel->giveDomain(di);
        int etype = 0, nnpe = 0, ndim = 3;
        for ( auto &el : d->giveElements() ) {
            int t = dynamic_cast< LSpace * >( el.get() ) ? OGB_LSPACE :
                    dynamic_cast< LTRSpace * >( el.get() ) ? OGB_LTRSPACE :
                    dynamic_cast< PlaneStress2d * >( el.get() ) ? OGB_PLANESTRESS2D : 0;
            if ( !t || ( etype && t != etype ) ) {
                return false;
            }
            etype = t;
            if ( !dynamic_cast< IsotropicLinearElasticMaterial * >( el->giveMaterial() ) ) {
                return false;
            }
        }
        if ( !etype ) {
            return false;
        }
        nnpe = etype == OGB_LSPACE ? 8 : 4;
        ndim = etype == OGB_PLANESTRESS2D ? 2 : 3;
        const int ndofpn = etype == OGB_PLANESTRESS2D ? 2 : 3;
        int nn = d->giveNumberOfDofManagers(), ne = d->giveNumberOfElements();
        std::vector< double >coords( ( size_t ) nn * ndim );
        std::vector< uint8_t >bc( ( size_t ) nn * ndofpn, 0 );
        TimeStep *tStep = eModel->giveCurrentStep();
        for ( int i = 1; i <= nn; i++ ) {
            DofManager *dm = d->giveDofManager(i);
            const FloatArray &x = dm->giveCoordinates();
            for ( int k = 0; k < ndim; k++ ) {
                coords [ ( size_t ) ( i - 1 ) * ndim + k ] = x [ k ];
            }
            int k = 0;
            for ( Dof *dof : *dm ) {
                if ( k < ndofpn ) {
                    bc [ ( size_t ) ( i - 1 ) * ndofpn + k ] = dof->hasBc(tStep) ? 1 : 0;
                }
                k++;
            }
        }
        std::vector< int >conn( ( size_t ) ne * nnpe ), emat(ne);
        std::vector< double >mats;
        std::map< Material *, int >matIndex;
        double thickness = 1.0;
        for ( int e = 1; e <= ne; e++ ) {
            Element *el = d->giveElement(e);
            for ( int a = 1; a <= nnpe; a++ ) {
                conn [ ( size_t ) ( e - 1 ) * nnpe + a - 1 ] = el->giveDofManagerNumber(a) - 1;
            }
            Material *mat = el->giveMaterial();
            auto it = matIndex.find(mat);
            if ( it == matIndex.end() ) {
                auto *iso = static_cast< IsotropicLinearElasticMaterial * >( mat );
                double row[8] = { ( double ) OGB_MAT_ISOLE, iso->giveYoungsModulus(), iso->givePoissonsRatio(), 0, 0, 0, 0, 0 };
                mats.insert(mats.end(), row, row + 8);
                it = matIndex.emplace(mat, ( int ) matIndex.size() ).first;
            }
            emat [ e - 1 ] = it->second;
            if ( etype == OGB_PLANESTRESS2D ) {
                thickness = el->giveCrossSection()->give(CS_Thickness, el->giveDefaultIntegrationRulePtr()->getIntegrationPoint(0) );
            }
        }
        gb300_check(ogb_model_create(gb300_context(), etype, nn, coords.data(), ne, conn.data(), emat.data(),
                                     ( int ) matIndex.size(), mats.data(), thickness, bc.data(), & model), "ogb_model_create");
        eqCache.assign( ( size_t ) nn * ndofpn, 0 );
        gb300_check(ogb_model_equations(model, eqCache.data() ), "ogb_model_equations");
        if ( !numberingMatches(eModel, di) ) {
            OOFEM_LOG_INFO("GpuCsrMtrx: equation numbering differs from the device's, host element loop used\n");
            dropDeviceElements();
            return false;
        }
        gb300_check(ogb_model_build_matrix(model, m), "ogb_model_build_matrix");
        emodel = eModel;
        domainIndex = di;
        return true;
    }

public:
    GpuCsrMtrx() : SparseMtrx()
    {
        OOFEM_LOG_INFO("GpuCsrMtrx: constructed by the class factory (smtype 11)\n");
        gb300_check(ogb_mtrx_create(gb300_context(), & m), "ogb_mtrx_create");
    }
    ~GpuCsrMtrx() override
    {
        dropDeviceElements();
        ogb_mtrx_destroy(m);
    }

    ogb_mtrx *handle() const { flush(); return m; }
    bool deviceElements() const { return model != nullptr; }

    // SparseMtrx::buildInternalStructure (sparsemtrx.h:198; CompCol compcol.C:174-272)
    int buildInternalStructure(EngngModel *eModel, int di, const UnknownNumberingScheme &s) override
    {
        Domain *d = eModel->giveDomain(di);
        int neq = eModel->giveNumberOfDomainEquations(di, s);
        nRows = nColumns = neq;
        pending.clear();
        dropDeviceElements();
        if ( s.isDefault() && tryDeviceElements(eModel, di) ) {
            // LinearStatic assembles right after building the structure
            if ( std::string(eModel->giveClassName() ) == "LinearStatic" ) {
                g_device_assembly = this;
            }
            this->version++;
            return 1;
        }
        std::vector< int64_t >ptr(1, 0);
        std::vector< int >loc;
        IntArray l;
        for ( auto &el : d->giveElements() ) {
            el->giveLocationArray(l, s);
            for ( int v : l ) {
                loc.push_back(v);
            }
            ptr.push_back( ( int64_t ) loc.size() );
        }
        gb300_check(ogb_mtrx_build_structure(m, neq, ( int ) ptr.size() - 1, ptr.data(), loc.data() ), "buildInternalStructure");
        this->version++;
        return 1;
    }

    // SparseMtrx::assemble (sparsemtrx.h:220); FloatMatrix storage is column-major
    int assemble(const IntArray &loc, const FloatMatrix &mat) override
    {
        if ( mat.giveNumberOfRows() == 0 ) {
            return 1;
        }
        std::vector< int >l(loc.begin(), loc.end() );
        return ogb_mtrx_assemble(m, ( int ) l.size(), l.data(), mat.givePointer() ) == OGB_OK ? 1 : 0;
    }

    int assemble(const IntArray &rloc, const IntArray &cloc, const FloatMatrix &mat) override
    {
        OOFEM_ERROR("GpuCsrMtrx: rectangular assembly is not supported");
        return 0;
    }

    int assembleBegin() override
    {
        flush();
        return ogb_mtrx_assemble_begin(m) == OGB_OK;
    }

    // SparseMtrx::assembleEnd (sparsemtrx.h:236), called once after every
    // EngngModel::assemble (engngm.C:1035-1036): the device launch hook.
    int assembleEnd() override
    {
        const bool device = model && g_device_assembly == this;
        if ( g_device_assembly == this ) {
            g_device_assembly = nullptr;
        }
        int r;
        if ( device ) {
            // the numbering may have moved since the structure was built (a boundary
            // condition switched on or off): rebuild the device mesh from the current
            // state, and refuse to go on if it still does not match OOFEM's
            if ( !numberingMatches(emodel, domainIndex) ) {
                dropDeviceElements();
                if ( !tryDeviceElements(emodel, domainIndex) ) {
                    OOFEM_ERROR("GpuCsrMtrx: equation numbering changed and the device mesh cannot follow it");
                }
            }
            r = ogb_model_assemble_stiffness(model, m);
        } else {
            r = ogb_mtrx_assemble_end(m);
        }
        gb300_check(r, "assembleEnd");
        this->version++;
        return 1;
    }

    void zero() override
    {
        pending.clear();
        gb300_check(ogb_mtrx_zero(m), "zero");
        if ( model ) {
            g_device_assembly = this;   // the drivers zero the matrix right before assembling it
        }
        this->version++;
    }

    void times(const FloatArray &x, FloatArray &answer) const override
    {
        flush();
        int neq = 0;
        gb300_check(ogb_mtrx_neq(m, & neq), "times");
        if ( x.giveSize() != nRows || neq != nRows ) {
            OOFEM_ERROR("GpuCsrMtrx::times: size mismatch");
        }
        answer.resize(nRows);
        gb300_check(ogb_mtrx_times(m, x.givePointer(), answer.givePointer() ), "times");
    }

    double &at(int i, int j) override
    {
        auto key = std::make_pair(i, j);
        auto it = pending.find(key);
        if ( it == pending.end() ) {
            double v = 0.0;
            gb300_check(ogb_mtrx_at(m, i, j, & v), "at");
            it = pending.emplace(key, v).first;
        }
        this->version++;
        return it->second;
    }

    double at(int i, int j) const override
    {
        auto it = pending.find(std::make_pair(i, j) );
        if ( it != pending.end() ) {
            return it->second;
        }
        double v = 0.0;
        gb300_check(ogb_mtrx_at(m, i, j, & v), "at");
        return v;
    }

    // LDLTFactorization (lstype 0, ldltfact.C:50-63) on this matrix: the device
    // L D L^T of the upper triangle (as Skyline::factorized, skyline.C:429-491),
    // kept until the next mutation; backSubstitutionWith solves with it.
    bool canBeFactorized() const override { return true; }
    SparseMtrx *factorized() override
    {
        gb300_check(ogb_ldlt_factorize(handle() ), "GpuCsrMtrx::factorized");
        return this;
    }
    FloatArray *backSubstitutionWith(FloatArray &y) const override
    {
        if ( y.giveSize() != nRows ) {
            OOFEM_ERROR("GpuCsrMtrx::backSubstitutionWith: size mismatch");
        }
        FloatArray x(nRows);
        gb300_check(ogb_ldlt_solve(handle(), y.givePointer(), x.givePointer() ), "GpuCsrMtrx::backSubstitutionWith");
        y = x;
        return & y;
    }
    SparseMtrxType giveType() const override { return SMT_GpuCsr; }
    bool isAsymmetric() const override { return false; }
    const char *giveClassName() const override { return "GpuCsrMtrx"; }
};

REGISTER_SparseMtrx(GpuCsrMtrx, SMT_GpuCsr);

/// Jacobi-PCG on the GPU (IML CG + DiagPreconditioner semantics), optionally the
/// mixed-precision form (gpuprec 1).
class GpuPcgSolver : public SparseLinearSystemNM
{
protected:
    double tol = 1.e-5;   // IMLSolver defaults (imlsolver.C:66-98)
    int maxite = 200;
    int precision = OGB_PREC_FP64;
    // IMLSolver's lsprecond numbering (imlsolver.C:78-94): 0 none, 1 diagonal,
    // 4 incomplete Cholesky. The default is the diagonal one, this solver's
    // Jacobi-PCG; IMLSolver's own default is 0 (no preconditioner).
    int precond = 1;

public:
    GpuPcgSolver(Domain *d, EngngModel *m) : SparseLinearSystemNM(d, m) { }

    void initializeFrom(InputRecord &ir) override
    {
        IR_GIVE_OPTIONAL_FIELD(ir, tol, _IFT_GpuPcgSolver_lstol);
        IR_GIVE_OPTIONAL_FIELD(ir, maxite, _IFT_GpuPcgSolver_lsiter);
        IR_GIVE_OPTIONAL_FIELD(ir, precision, _IFT_GpuPcgSolver_gpuprec);
        IR_GIVE_OPTIONAL_FIELD(ir, precond, _IFT_GpuPcgSolver_lsprecond);
    }

    ConvergedReason solve(SparseMtrx &A, FloatArray &b, FloatArray &x) override
    {
        auto *g = dynamic_cast< GpuCsrMtrx * >( & A );
        if ( !g ) {
            OOFEM_ERROR("GpuPcgSolver needs a GpuCsrMtrx (smtype 11)");
        }
        int neq = 0;
        if ( ogb_mtrx_neq(g->handle(), & neq) != OGB_OK || b.giveSize() != A.giveNumberOfRows() || neq != b.giveSize() ) {
            OOFEM_ERROR("GpuPcgSolver: right-hand side of %d entries for a matrix of %d equations",
                        b.giveSize(), A.giveNumberOfRows() );
        }
        if ( x.giveSize() != b.giveSize() ) {
            x.resize(b.giveSize() );
            x.zero();
        }
        ogb_solve_info info;
        if ( ogb_mtrx_set_preconditioner(g->handle(), precond) != OGB_OK ) {
            OOFEM_ERROR("GpuPcgSolver: %s", ogb_last_error());
        }
        int r = ogb_pcg_solve(g->handle(), b.givePointer(), x.givePointer(), tol, maxite, precision, & info);
        OOFEM_LOG_INFO("GpuPcg(%s): status %d, nite %d, achieved tol. %g\n",
                       precision == OGB_PREC_MIXED ? "mixed" : "fp64", info.status, info.iterations, info.achieved);
        if ( r == OGB_OK ) {
            return CR_CONVERGED;
        }
        if ( r == OGB_E_NOTCONV ) {
            return CR_DIVERGED_ITS;
        }
        return CR_FAILED;
    }

    /// Multiple right-hand sides (sparselinsystemnm.h:91): one batched solve on the
    /// device instead of the default column loop (sparselinsystemnm.C:47-69).
    ConvergedReason solve(SparseMtrx &A, FloatMatrix &B, FloatMatrix &X) override
    {
        auto *g = dynamic_cast< GpuCsrMtrx * >( & A );
        if ( !g ) {
            OOFEM_ERROR("GpuPcgSolver needs a GpuCsrMtrx (smtype 11)");
        }
        const int neq = A.giveNumberOfRows(), nrhs = B.giveNumberOfColumns();
        if ( B.giveNumberOfRows() != neq ) {
            OOFEM_ERROR("A and B matrix mismatch");
        }
        if ( X.giveNumberOfRows() != neq || X.giveNumberOfColumns() != nrhs ) {
            X.resize(neq, nrhs);
        }
        if ( ogb_mtrx_set_preconditioner(g->handle(), precond) != OGB_OK ) {
            OOFEM_ERROR("GpuPcgSolver: %s", ogb_last_error());
        }
        std::vector< int > iters(nrhs), status(nrhs);
        std::vector< double > achieved(nrhs);
        int r = ogb_pcg_solve_multi(g->handle(), nrhs, B.givePointer(), X.givePointer(), tol, maxite, precision,
                                    iters.data(), achieved.data(), status.data());
        for ( int c = 0; c < nrhs; ++c ) {
            OOFEM_LOG_INFO("GpuPcg(%s) rhs %d: status %d, nite %d, achieved tol. %g\n",
                           precision == OGB_PREC_MIXED ? "mixed" : "fp64", c + 1, status [ c ], iters [ c ],
                           achieved [ c ]);
        }
        if ( r == OGB_OK ) {
            return CR_CONVERGED;
        }
        if ( r == OGB_E_NOTCONV ) {
            return CR_DIVERGED_ITS;
        }
        return CR_FAILED;
    }

    LinSystSolverType giveLinSystSolverType() const override { return ST_GpuPcg; }
    SparseMtrxType giveRecommendedMatrix(bool symmetric) const override { return SMT_GpuCsr; }
    const char *giveClassName() const override { return "GpuPcgSolver"; }
};

REGISTER_SparseLinSolver(GpuPcgSolver, ST_GpuPcg);

// GPU element backend: the same keywords as the reference elements, registered
// after them so they take over for an unchanged input file (classfactory.C:128-133
// stores the latest creator). While a GpuCsrMtrx assembles on the device (the
// window of g_device_assembly) the stiffness handed to the host loop is empty;
// everything else (internal forces, the extrapolated forces of IG_Tangent, output,
// context) is the reference element's.
#define GB300_DEVICE_ELEMENT(NAME, BASE, KEYWORD)                                              \
    class NAME : public BASE                                                                    \
    {                                                                                           \
    public:                                                                                     \
        NAME(int n, Domain *d) : BASE(n, d) { }                                                 \
        void computeStiffnessMatrix(FloatMatrix &answer, MatResponseMode rMode, TimeStep *tStep) override \
        {                                                                                       \
            if ( g_device_assembly ) {                                                          \
                answer.clear();                                                                 \
                return;                                                                         \
            }                                                                                   \
            BASE::computeStiffnessMatrix(answer, rMode, tStep);                                 \
        }                                                                                       \
        const char *giveInputRecordName() const override { return KEYWORD; }                    \
    };

GB300_DEVICE_ELEMENT(GpuLSpace, LSpace, "lspace")
GB300_DEVICE_ELEMENT(GpuLTRSpace, LTRSpace, "ltrspace")
GB300_DEVICE_ELEMENT(GpuPlaneStress2d, PlaneStress2d, "planestress2d")

#define _IFT_GpuLSpace_Name "lspace"
#define _IFT_GpuLTRSpace_Name "ltrspace"
#define _IFT_GpuPlaneStress2d_Name "planestress2d"
REGISTER_Element(GpuLSpace)
REGISTER_Element(GpuLTRSpace)
REGISTER_Element(GpuPlaneStress2d)

} // end namespace oofem
