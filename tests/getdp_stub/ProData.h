/* Stand-in for GetDP's ProData.h: nothing the backend uses beyond
   DofData.h.  Test infrastructure. */
#ifndef PRODATA_STUB_H
#define PRODATA_STUB_H
#include "DofData.h"
#endif
