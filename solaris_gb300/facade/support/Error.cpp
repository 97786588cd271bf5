// Standalone Error: last message and the location stack.
#include "Error.h"

#include <cstdio>

std::string Error::_errMsg;
std::list<std::string> Error::_stackTrace;

void Error::PushLocation(const char* file, const char* function, long line) {
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s:%s:%ld", file, function, line);
  _stackTrace.push_back(buf);
}

void Error::PrintStackTrace() {
  for (const std::string& s : _stackTrace) std::fprintf(stderr, "\t%s\n", s.c_str());
}
