/* Stand-in for GetDP's MallocUtils.h (Malloc / Free).  Test infrastructure. */
#ifndef MALLOCUTILS_STUB_H
#define MALLOCUTILS_STUB_H
#include <stddef.h>
void *Malloc(size_t size);
void Free(void *ptr);
#endif
