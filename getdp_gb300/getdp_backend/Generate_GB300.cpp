// The batched Generate hook of the GB300 backend.
//
// GetDP's element loop (Treatment_FemFormulation,
// src/kernel/Treatment_Formulation.cpp:413-618) evaluates every Galerkin term
// element by element (Cal_GalerkinTermOfFemEquation,
// Cal_GalerkinTermOfFemEquation.cpp:531-1014) and adds each local entry with
// LinAlg_AddDoubleInMatrix.  For the terms this backend's element kernels
// evaluate, the hook gathers, once per Generate and before the loop, the
// element tables the kernels need -- node coordinates, the unknown numbers
// of the element's DOFs in GetDP's numbering (fixed DOFs with their values),
// one coefficient per element -- and submits them as one term batch
// (gb300_generate_pattern / gb300_generate_values); the loop then skips those
// (term, element) pairs and evaluates everything else as before.
//
// Terms taken (all others stay on the CPU path):
//   [ c[] * Dof{d a}, {d a} ] or [ Dof{d a}, {d a} ]   (CWQ_EXP_TIME_DOF, CWQ_DOF)
//   with a and its test function the same quantity, BF_PerpendicularEdge or
//   BF_Node on 3-node triangles, no time derivative, Jacobian Vol, 3-point
//   Gauss, one harmonic.  c[] must be constant on the element (it is
//   evaluated at the three Gauss points; an element where it varies, or of
//   another type, or with a DOF that is neither unknown nor fixed, is left to
//   the CPU).  The 2D curl-curl of BF_PerpendicularEdge and the Laplacian of
//   BF_Node give the same element matrix, c grad N_i . grad N_j.
// The hook is active only on a matrix nothing else has been added to since
// it was created (GetDP's ZeroMatrix before Generate), so that the batch's
// pattern is A's whole pattern; entries the CPU path adds later are merged
// by LinAlg_AssembleMatrix.
//
// GB300_GENERATE_DUMP=<file> writes the gathered batch (binary: counts, then
// the arrays) before it is submitted, for checking the gather without a GPU.

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <set>
#include <utility>
#include <vector>

#include "GetDPConfig.h"

#if defined(HAVE_GB300)

#include "BF.h"
#include "Cal_AssembleTerm.h"
#include "Cal_Quantity.h"
#include "DofData.h"
#include "ExtendedGroup.h"
#include "GeoData.h"
#include "Get_DofOfElement.h"
#include "Get_FunctionValue.h"
#include "Get_Geometry.h"
#include "LinAlg.h"
#include "ListUtils.h"
#include "Message.h"
#include "ProData.h"
#include "ProDefine.h"

extern struct Problem Problem_S;
extern struct CurrentData Current;

// LinAlg_GB300.cpp: nothing added to A since it was created or zeroed, and
// the GPU copy of b made current
int GB300_MatrixUntouched(gMatrix *A);
void GB300_VectorOnDevice(gVector *V);
void GB300_VectorDeviceWritten(gVector *V);

namespace {

std::vector<char> g_taken;                 // per equation term: the hook took it
std::set<std::pair<int, int> > g_left;     // (term, element number) left to the CPU

// the 3-point Gauss rule of Gauss_Triangle.h:13-16 (u, v)
const double kU3[3] = {0.16666666666666, 0.66666666666666, 0.16666666666666};
const double kV3[3] = {0.16666666666666, 0.16666666666666, 0.66666666666666};

bool term_form_ok(struct EquationTerm *T, struct QuantityStorage *QS0)
{
  if(T->Type != GALERKIN) return false;
  struct FemLocalTermActive *FI = T->Case.LocalTerm.Active;
  const auto &t = T->Case.LocalTerm.Term;
  if(!FI || FI->MHBilinear) return false;
  if(t.TypeTimeDerivative != NODT_) return false;
  if(t.DefineQuantityIndexEqu != t.DefineQuantityIndexDof ||
     t.DefineQuantityIndexEqu < 0)
    return false;
  if(t.TypeOperatorEqu != EXTDER || t.TypeOperatorDof != EXTDER) return false;
  if(t.CanonicalWholeQuantity != CWQ_DOF && t.CanonicalWholeQuantity != CWQ_EXP_TIME_DOF)
    return false;
  if(t.CanonicalWholeQuantity_Equ != CWQ_NONE) return false;
  if(T->Case.LocalTerm.SubRegion >= 0 || T->Case.LocalTerm.ExpressionIndexForMetricTensor >= 0)
    return false;
  for(int i = 0; i < t.NbrQuantityIndex; i++)
    if(t.QuantityTraceGroupIndexTable[i] >= 0) return false;
  if(FI->NbrJacobianCase != 1 || FI->JacobianCase_P0[0].TypeJacobian != JACOBIAN_VOL)
    return false;
  struct QuantityStorage *QS = QS0 + t.DefineQuantityIndexEqu;
  if(QS->DefineQuantity->Type != LOCALQUANTITY || !QS->FunctionSpace) return false;
  List_T *bfl = QS->FunctionSpace->BasisFunction;
  if(!bfl || List_Nbr(bfl) < 1) return false;
  for(int i = 0; i < List_Nbr(bfl); i++) {
    struct BasisFunction *bf = (struct BasisFunction *)List_Pointer(bfl, i);
    if(bf->Function != (void (*)())BF_PerpendicularEdge &&
       bf->Function != (void (*)())BF_Node)
      return false;
  }
  return true;
}

// the term's integration rule on this element is the 3-point Gauss rule
bool gauss3(struct Element *E, struct EquationTerm *T)
{
  struct FemLocalTermActive *FI = T->Case.LocalTerm.Active;
  struct IntegrationCase *IC =
    Get_IntegrationCase(E, FI->IntegrationCase_L, FI->CriterionIndex);
  if(!IC || IC->Type != GAUSS) return false;
  for(int k = 0; k < List_Nbr(IC->Case); k++) {
    struct Quadrature *Q = (struct Quadrature *)List_Pointer(IC->Case, k);
    if(Q->ElementType == TRIANGLE) return Q->NumberOfPoints == 3;
  }
  return false;
}

struct Gathered {
  std::vector<double> nodes;  // 3 x 3 per element (x, y, z of its 3 nodes)
  std::vector<int> elems, edofs;
  std::vector<double> coef, fixed;
};

// gathers one (term, element); false when the element must stay on the CPU
bool gather(struct Element *E, struct EquationTerm *T, struct QuantityStorage *QS0,
            Gathered &G)
{
  const auto &t = T->Case.LocalTerm.Term;
  struct QuantityStorage *QS = QS0 + t.DefineQuantityIndexEqu;
  if(E->Type != TRIANGLE || E->GeoElement->NbrNodes != 3 || !gauss3(E, T)) return false;
  QS->NumLastElementForFunctionSpace = E->Num;
  Get_DofOfElement(E, QS->FunctionSpace, QS, QS->DefineQuantity->IndexInFunctionSpace);
  if(QS->NbrElementaryBasisFunction != 3) return false;
  Get_NodesCoordinatesOfElement(E);
  int d[3];
  double g[3] = {0., 0., 0.};
  int nf = 0;
  for(int k = 0; k < 3; k++) {
    struct Dof *D = QS->BasisFunction[k].Dof;
    if(QS->BasisFunction[k].NumEntityInElement != k) return false;  // node k of the element
    if(D->Type == DOF_UNKNOWN)
      d[k] = D->Case.Unknown.NumDof - 1;
    else if(D->Type == DOF_FIXED) {
      double v = 0.;
      LinAlg_GetDoubleInScalar(&v, &D->Val);
      g[k] = v * Current.DofData->CurrentSolution
                   ->TimeFunctionValues[D->Case.FixedAssociate.TimeFunctionIndex];
      d[k] = -1;  // numbered below
      nf++;
    }
    else
      return false;
  }
  // the coefficient, at the three Gauss points (it must not vary)
  double c = 1.;
  if(t.CanonicalWholeQuantity == CWQ_EXP_TIME_DOF) {
    struct Expression *X =
      (struct Expression *)List_Pointer(Problem_S.Expression, t.ExpressionIndexForCanonical);
    Current.Element = E;
    for(int q = 0; q < 3; q++) {
      double u = kU3[q], v = kV3[q];
      double n[3] = {1. - u - v, u, v};
      Current.x = Current.y = Current.z = 0.;
      for(int k = 0; k < 3; k++) {
        Current.x += n[k] * E->x[k];
        Current.y += n[k] * E->y[k];
        Current.z += n[k] * E->z[k];
      }
      Current.u = u;
      Current.v = v;
      Current.w = 0.;
      struct Value V;
      Get_ValueOfExpression(X, QS0, u, v, 0., &V);
      if(V.Type != SCALAR) return false;
      if(q == 0)
        c = V.Val[0];
      else if(V.Val[0] != c)
        return false;
    }
  }
  const int e = (int)G.coef.size();
  for(int k = 0; k < 3; k++) {
    G.nodes.push_back(E->x[k]);
    G.nodes.push_back(E->y[k]);
    G.nodes.push_back(E->z[k]);
    G.elems.push_back(3 * e + k);
    if(d[k] >= 0)
      G.edofs.push_back(d[k]);
    else {
      G.edofs.push_back(-1 - (int)G.fixed.size());
      G.fixed.push_back(g[k]);
    }
  }
  G.coef.push_back(c);
  (void)nf;
  return true;
}

void dump(const char *path, const Gathered &G)
{
  FILE *f = fopen(path, "wb");
  if(!f) return;
  int ne = (int)G.coef.size(), nfx = (int)G.fixed.size();
  fwrite(&ne, sizeof(int), 1, f);
  fwrite(&nfx, sizeof(int), 1, f);
  fwrite(G.nodes.data(), sizeof(double), G.nodes.size(), f);
  fwrite(G.edofs.data(), sizeof(int), G.edofs.size(), f);
  fwrite(G.coef.data(), sizeof(double), G.coef.size(), f);
  fwrite(G.fixed.data(), sizeof(double), G.fixed.size(), f);
  fclose(f);
}

}  // namespace

// Before the element loop of a STATUS_CAL Treatment_FemFormulation (the terms
// initialised): gathers and submits the terms the hook takes.  Returns 1 when
// the loop must ask GB300_Generate_Skip before each Galerkin evaluation.
int GB300_Generate_Begin(struct EquationTerm *EquationTerm_P0, int Nbr_EquationTerm,
                         struct QuantityStorage *QuantityStorage_P0,
                         struct Group *Generate_Group)
{
  g_taken.assign(Nbr_EquationTerm, 0);
  g_left.clear();
  if(getenv("GB300_NO_GENERATE_HOOK")) return 0;
  if(Current.NbrHar != 1 || Current.DofData->Flag_Only || Current.DofData->Flag_RHS ||
     Current.TypeAssembly == ASSEMBLY_SEPARATE)
    return 0;
  gMatrix *A = &Current.DofData->A;
  gVector *b = &Current.DofData->b;
  if(!GB300_MatrixUntouched(A)) return 0;
  int any = 0;
  for(int i = 0; i < Nbr_EquationTerm; i++)
    if(term_form_ok(EquationTerm_P0 + i, QuantityStorage_P0)) {
      g_taken[i] = 1;
      any = 1;
    }
  if(!any) return 0;

  Gathered G;
  struct Element Element;
  const int Nbr_Element = Geo_GetNbrGeoElements();
  for(int i_Element = 0; i_Element < Nbr_Element; i_Element++) {
    Element.GeoElement = Geo_GetGeoElement(i_Element);
    Element.Region = Element.GeoElement->Region;
    if(Generate_Group &&
       !List_Search(Generate_Group->InitialList, &Element.Region, fcmp_int))
      continue;
    Element.Num = Element.GeoElement->Num;
    Element.Type = Element.GeoElement->Type;
    Current.Region = Element.Region;
    for(int i = 0; i < Nbr_EquationTerm; i++) {
      if(!g_taken[i]) continue;
      struct EquationTerm *T = EquationTerm_P0 + i;
      struct Group *In =
        (struct Group *)List_Pointer(Problem_S.Group, T->Case.LocalTerm.InIndex);
      bool in = (In->Type != ELEMENTLIST &&
                 List_Search(In->InitialList, &Element.Region, fcmp_int)) ||
                (In->Type == ELEMENTLIST &&
                 Check_IsEntityInExtendedGroup(In, Element.Num, 0));
      if(!in) continue;
      Current.IntegrationSupportIndex = T->Case.LocalTerm.InIndex;
      if(!gather(&Element, T, QuantityStorage_P0, G))
        g_left.insert(std::make_pair(i, Element.Num));
    }
  }
  const int ne = (int)G.coef.size();
  if(const char *path = getenv("GB300_GENERATE_DUMP")) dump(path, G);
  if(ne == 0) {
    for(auto &t : g_taken) t = 0;
    return 0;
  }
  gb300_term_batch tb;
  memset(&tb, 0, sizeof(tb));
  tb.kind = GB300_TERM_TRI3_MAGNETOSTATIC;
  tb.n_nodes = 3 * ne;
  tb.n_elems = ne;
  tb.nodes = G.nodes.data();
  tb.elems = G.elems.data();
  tb.elem_dofs = G.edofs.data();
  tb.coef = G.coef.data();
  tb.fixed_values = G.fixed.empty() ? nullptr : G.fixed.data();
  tb.n_fixed = (int)G.fixed.size();
  tb.scatter = GB300_SCATTER_DEFAULT;
  if(gb300_generate_pattern(A->M, &tb) != GB300_OK) {
    Message::Error("GB300 backend: %s", gb300_last_error());
    return 0;
  }
  GB300_VectorOnDevice(b);
  if(gb300_generate_values(A->M, b->D, &tb) != GB300_OK) {
    Message::Error("GB300 backend: %s", gb300_last_error());
    return 0;
  }
  GB300_VectorDeviceWritten(b);
  Message::Info("GB300 backend: %d element matrices assembled on the GPU", ne);
  return 1;
}

// true when the term's batch already holds this element's contribution
int GB300_Generate_Skip(int i_EquTerm, int element_num)
{
  if(i_EquTerm < 0 || i_EquTerm >= (int)g_taken.size() || !g_taken[i_EquTerm]) return 0;
  return g_left.count(std::make_pair(i_EquTerm, element_num)) ? 0 : 1;
}

#endif
