// Definitions behind the stand-in headers: Message, Malloc/Free, Current
// and Name_Path.  Test infrastructure (see LinAlg.h in this folder).
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>

#include "DofData.h"
#include "MallocUtils.h"
#include "Message.h"

static struct DofData g_dofdata = {nullptr};
struct CurrentData Current = {&g_dofdata};
char *Name_Path = (char *)"";

static void vprint(const char *tag, const char *fmt, va_list ap)
{
  fprintf(stderr, "%s: ", tag);
  vfprintf(stderr, fmt, ap);
  fprintf(stderr, "\n");
}

void Message::Error(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vprint("Error", fmt, ap);
  va_end(ap);
  exit(1);
}
void Message::Warning(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vprint("Warning", fmt, ap);
  va_end(ap);
}
void Message::Info(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vprint("Info", fmt, ap);
  va_end(ap);
}

void *Malloc(size_t size)
{
  void *p = malloc(size ? size : 1);
  if(!p) Message::Error("out of memory (%zu bytes)", size);
  return p;
}
void Free(void *p) { free(p); }
