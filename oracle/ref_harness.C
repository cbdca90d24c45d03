// Reference harness -- TEST INFRASTRUCTURE ONLY.
//
// Links against a build of the reference (liboofem) and runs an unchanged OOFEM
// input deck, adding one export module, "refdump", that writes full-precision
// (%.17g) per-step data the .out file only carries to 8 digits:
//   step <n> <target time> <Newton iterations of the step>
//   u <node> <dof> <eq> <value>             (eq: default numbering; 0 = prescribed)
//   gp <elem> <gp> s <stress...> e <strain...> k <kappa> w <omega> le <Le>
//   reac <node> <dof> <value>
// With "-K" the final tangent matrix is assembled into a CompCol and written as
//   K <neq> <nnz> / colptr ... / rowind ... / val ...
// and the first element stiffness matrices as "ke <elem> <n> <values row-major>".
//
// Usage: ref_harness -f deck.in -o dump.txt [-K]
// The generated files are turned into tests/golden fixtures by
// tests/golden/make_golden.py; nothing in the product uses this file.
#include "oofemtxtdatareader.h"
#include "engngm.h"
#include "util.h"
#include "exportmodule.h"
#include "classfactory.h"
#include "domain.h"
#include "dofmanager.h"
#include "dof.h"
#include "element.h"
#include "gausspoint.h"
#include "integrationrule.h"
#include "timestep.h"
#include "unknownnumberingscheme.h"
#include "compcol.h"
#include "assemblercallback.h"
#include "floatmatrix.h"
#include "sm/EngineeringModels/structengngmodel.h"
#include "sm/Materials/structuralms.h"
#include "sm/Materials/misesmat.h"
#include "sm/Materials/isodamagemodel.h"

#include <cstdio>
#include <cstring>
#include <string>

using namespace oofem;

static FILE *g_out = nullptr;

#define _IFT_RefDump_Name "refdump"

class RefDump : public ExportModule
{
public:
    RefDump(int n, EngngModel *e) : ExportModule(n, e) { }
    void doOutput(TimeStep *tStep, bool forcedOutput) override
    {
        // NRSolver also calls export modules with forcedOutput after every
        // iteration (nrsolver.C); only converged end-of-step states are dumped.
        if ( !g_out || forcedOutput ) {
            return;
        }
        Domain *d = emodel->giveDomain(1);
        EModelDefaultEquationNumbering num;
        fprintf(g_out, "step %d %.17g %d\n", tStep->giveNumber(), tStep->giveTargetTime(), tStep->numberOfIterations);
        for ( auto &node : d->giveDofManagers() ) {
            for ( Dof *dof : *node ) {
                fprintf(g_out, "u %d %d %d %.17g\n", node->giveNumber(), ( int ) dof->giveDofID(),
                        dof->giveEquationNumber(num), dof->giveUnknown(VM_Total, tStep));
            }
        }
        for ( auto &el : d->giveElements() ) {
            IntegrationRule *ir = el->giveDefaultIntegrationRulePtr();
            for ( GaussPoint *gp : *ir ) {
                auto *ms = dynamic_cast< StructuralMaterialStatus * >( gp->giveMaterialStatus() );
                if ( !ms ) {
                    continue;
                }
                fprintf(g_out, "gp %d %d s", el->giveNumber(), gp->giveNumber());
                for ( double v : ms->giveStressVector() ) {
                    fprintf(g_out, " %.17g", v);
                }
                fprintf(g_out, " e");
                for ( double v : ms->giveStrainVector() ) {
                    fprintf(g_out, " %.17g", v);
                }
                double k = 0, w = 0, le = 0;
                if ( auto *mm = dynamic_cast< MisesMatStatus * >( ms ) ) {
                    k = mm->giveCumulativePlasticStrain();
                    w = mm->giveDamage();
                } else if ( auto *dm = dynamic_cast< IsotropicDamageMaterialStatus * >( ms ) ) {
                    k = dm->giveKappa();
                    w = dm->giveDamage();
                    le = dm->giveLe();
                }
                fprintf(g_out, " k %.17g w %.17g le %.17g\n", k, w, le);
            }
        }
        if ( auto *sem = dynamic_cast< StructuralEngngModel * >( emodel ) ) {
            FloatArray reactions;
            IntArray dofManMap, dofidMap, eqnMap;
            sem->buildReactionTable(dofManMap, dofidMap, eqnMap, tStep, 1);
            sem->computeReaction(reactions, tStep, 1);
            for ( int i = 1; i <= dofManMap.giveSize(); i++ ) {
                fprintf(g_out, "reac %d %d %.17g\n", dofManMap.at(i), dofidMap.at(i), reactions.at(eqnMap.at(i) ));
            }
        }
        fflush(g_out);
    }
    const char *giveClassName() const override { return "RefDump"; }
    const char *giveInputRecordName() const { return _IFT_RefDump_Name; }
};

REGISTER_ExportModule(RefDump)

int main(int argc, char **argv)
{
    std::string deck, out;
    bool dumpK = false;
    for ( int i = 1; i < argc; i++ ) {
        if ( !strcmp(argv [ i ], "-f") && i + 1 < argc ) {
            deck = argv [ ++i ];
        } else if ( !strcmp(argv [ i ], "-o") && i + 1 < argc ) {
            out = argv [ ++i ];
        } else if ( !strcmp(argv [ i ], "-K") ) {
            dumpK = true;
        }
    }
    if ( deck.empty() || out.empty() ) {
        fprintf(stderr, "usage: ref_harness -f deck.in -o dump.txt [-K]\n");
        return 2;
    }
    g_out = fopen(out.c_str(), "w");
    if ( !g_out ) {
        return 3;
    }
    OOFEMTXTDataReader dr(deck);
    auto problem = InstanciateProblem(dr, _processor, 0, nullptr, false);
    if ( !problem ) {
        return 4;
    }
    problem->checkProblemConsistency();
    problem->init();
    problem->solveYourself();

    if ( dumpK ) {
        TimeStep *tStep = problem->giveCurrentStep();
        Domain *d = problem->giveDomain(1);
        EModelDefaultEquationNumbering num;
        CompCol K;
        K.buildInternalStructure(problem.get(), 1, num);
        problem->assemble(K, tStep, TangentAssembler(TangentStiffness), num, d);
        int neq = K.giveNumberOfRows();
        const IntArray &colptr = K.giveColPtr();
        const IntArray &rowind = K.giveRowIndex();
        const FloatArray &val = K.giveValues();
        fprintf(g_out, "K %d %d\ncolptr", neq, rowind.giveSize());
        for ( int v : colptr ) {
            fprintf(g_out, " %d", v);
        }
        fprintf(g_out, "\nrowind");
        for ( int v : rowind ) {
            fprintf(g_out, " %d", v);
        }
        fprintf(g_out, "\nval");
        for ( double v : val ) {
            fprintf(g_out, " %.17g", v);
        }
        fprintf(g_out, "\n");
        int nke = d->giveNumberOfElements() < 4 ? d->giveNumberOfElements() : 4;
        for ( int e = 1; e <= nke; e++ ) {
            FloatMatrix ke;
            d->giveElement(e)->giveCharacteristicMatrix(ke, TangentStiffnessMatrix, tStep);
            fprintf(g_out, "ke %d %d", e, ke.giveNumberOfRows());
            for ( int i = 1; i <= ke.giveNumberOfRows(); i++ ) {
                for ( int j = 1; j <= ke.giveNumberOfColumns(); j++ ) {
                    fprintf(g_out, " %.17g", ke.at(i, j));
                }
            }
            fprintf(g_out, "\n");
        }
    }
    fclose(g_out);
    return 0;
}
