/* Stand-in for the parts of GetDP's DofData.h / Current the backend reads:
   the DOF data's DummyDof mask (null: no dummy DOFs).  Test infrastructure. */
#ifndef DOFDATA_STUB_H
#define DOFDATA_STUB_H
struct DofData {
  int *DummyDof;
};
struct CurrentData {
  struct DofData *DofData;
};
#endif
