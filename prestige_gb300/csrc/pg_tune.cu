// Autotuner (placeholder until the tuned variants land).
#include "pg_system.cuh"
extern "C" {
int pg_autotune(pg_system*, int, int*, double*, int*, double*) { pg::set_error("not built"); return PG_ESTATE; }
}
