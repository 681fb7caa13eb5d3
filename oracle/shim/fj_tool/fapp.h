/* Test infrastructure (oracle build only): stands in for the Fujitsu profiler
 * header that the reference's solver.h includes unconditionally
 * (src/solver.h:25-29).  The region calls become no-ops. */
#ifndef HBICG_ORACLE_FAPP_SHIM_H
#define HBICG_ORACLE_FAPP_SHIM_H
#define fapp_start(name, num, level) ((void)0)
#define fapp_stop(name, num, level) ((void)0)
#endif
