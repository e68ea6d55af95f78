/* Stand-in for GetDP's Message class (src/common/Message.h): what the
   backend calls.  Error prints "Error   : ..." and ends the program with
   status 1, as GetDP does on the command line; Info and Warning print to
   stderr.  Test infrastructure. */
#ifndef MESSAGE_STUB_H
#define MESSAGE_STUB_H
class Message {
public:
  static void Error(const char *fmt, ...);
  static void Warning(const char *fmt, ...);
  static void Info(const char *fmt, ...);
};
#endif
