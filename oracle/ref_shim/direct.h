#pragma once
// MSVC directory and conversion helpers the reference's output writers use.
#include <stdio.h>
#include <sys/stat.h>
#define _mkdir(p) mkdir((p), 0755)
static inline char* _itoa(int value, char* buf, int radix) {
  (void)radix;  // the reference converts in base 10 only
  sprintf(buf, "%d", value);
  return buf;
}
