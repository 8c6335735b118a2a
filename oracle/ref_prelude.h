/*
 * ref_prelude.h - force-included ahead of the reference's own headers when
 * oracle/Makefile builds oracle/_ref/libamt_ref.so.  TEST INFRASTRUCTURE.
 *
 * The reference reads its cache geometry with sysconf(_SC_LEVEL*_CACHE_*)
 * (include/cache_manager.hpp:107-150) and divides by the results
 * (include/mtm.hpp:45,57,69; include/mtv.hpp:33-37).  glibc can report 0 for
 * those names (notably on aarch64), so every sysconf call in the reference
 * translation unit is routed through a wrapper that falls back to sysfs.
 * The reference files themselves are compiled unmodified.
 */
#ifndef GBBLAS_REF_PRELUDE_H
#define GBBLAS_REF_PRELUDE_H
/* Standard headers the reference uses without including them itself
 * (std::cerr in include/utils.hpp:157, CHAR_BIT in include/cpuinfo.hpp:205,
 * std::ceil in include/mtm.hpp:78); a real Boost install pulls them in
 * transitively. */
#ifdef __cplusplus
#include <climits>
#include <cmath>
#include <iostream>
#include <sstream>
#endif
#include <stdio.h>
#include <string.h>
#include <unistd.h>

static inline long gbblas_ref_sysfs(int level, const char* leaf) {
  for (int idx = 0; idx < 8; ++idx) {
    char path[256], buf[64];
    snprintf(path, sizeof path, "/sys/devices/system/cpu/cpu0/cache/index%d/level", idx);
    FILE* f = fopen(path, "r");
    if (!f) continue;
    int lv = 0;
    if (fscanf(f, "%d", &lv) != 1) lv = 0;
    fclose(f);
    if (lv != level) continue;
    snprintf(path, sizeof path, "/sys/devices/system/cpu/cpu0/cache/index%d/type", idx);
    f = fopen(path, "r");
    if (!f) continue;
    buf[0] = 0;
    if (fscanf(f, "%63s", buf) != 1) buf[0] = 0;
    fclose(f);
    if (strcmp(buf, "Instruction") == 0) continue;
    snprintf(path, sizeof path, "/sys/devices/system/cpu/cpu0/cache/index%d/%s", idx, leaf);
    f = fopen(path, "r");
    if (!f) continue;
    long v = 0;
    char unit = 0;
    int got = fscanf(f, "%ld%c", &v, &unit);
    fclose(f);
    if (got >= 1) {
      if (got == 2 && (unit == 'K' || unit == 'k')) v *= 1024;
      if (got == 2 && (unit == 'M' || unit == 'm')) v *= 1024 * 1024;
      return v;
    }
  }
  return 0;
}

static inline long gbblas_ref_sysconf(int name) {
  long v = sysconf(name);
  if (v > 0) return v;
  switch (name) {
    case _SC_LEVEL1_DCACHE_SIZE: return gbblas_ref_sysfs(1, "size");
    case _SC_LEVEL2_CACHE_SIZE: return gbblas_ref_sysfs(2, "size");
    case _SC_LEVEL3_CACHE_SIZE: return gbblas_ref_sysfs(3, "size");
    case _SC_LEVEL1_DCACHE_ASSOC: return gbblas_ref_sysfs(1, "ways_of_associativity");
    case _SC_LEVEL2_CACHE_ASSOC: return gbblas_ref_sysfs(2, "ways_of_associativity");
    case _SC_LEVEL3_CACHE_ASSOC: return gbblas_ref_sysfs(3, "ways_of_associativity");
    case _SC_LEVEL1_DCACHE_LINESIZE: return gbblas_ref_sysfs(1, "coherency_line_size");
    case _SC_LEVEL2_CACHE_LINESIZE: return gbblas_ref_sysfs(2, "coherency_line_size");
    case _SC_LEVEL3_CACHE_LINESIZE: return gbblas_ref_sysfs(3, "coherency_line_size");
    default: return v;
  }
}
#define sysconf gbblas_ref_sysconf
#endif
