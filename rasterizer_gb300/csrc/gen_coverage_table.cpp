// Writes coverage_table.h: the 4096-entry coverage-mask table as built by
// coverage_table_build.h on this host.  Generated on x86-64, where it equals
// the table the reference builds at start-up.
//   g++ -O2 -ffp-contract=off gen_coverage_table.cpp -o gen && ./gen > coverage_table.h
#include <stdio.h>
#include "coverage_table_build.h"

int main()
{
  static int64_t t[4096];
  occ_table::build_coverage_table(t);
  printf("// Generated by gen_coverage_table.cpp (x86-64): 8x8 coverage masks indexed by\n"
         "// slope << 6 | offset.  Data, not code; layout in coverage_table_build.h.\n"
         "#pragma once\n#define OCC_COVERAGE_TABLE_VALUES \\\n");
  for (int i = 0; i < 4096; ++i)
    printf("0x%016llxull,%s", (unsigned long long)t[i], (i % 4 == 3) ? " \\\n" : "");
  printf("\n");
  return 0;
}
