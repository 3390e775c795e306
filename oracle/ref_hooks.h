// Shared state between ref_support.cpp and ref_driver.cpp (reference build
// only; test infrastructure).
#pragma once
#include <cstdio>
struct RefHooks {
  FILE* log;   // receives the reference's console report when non-null
  FILE* rec;   // receives one block of nodal state per recorded time
  long long padding[8];
};
extern RefHooks ref_hooks_storage;
void ref_record_state(int solution, double time);
