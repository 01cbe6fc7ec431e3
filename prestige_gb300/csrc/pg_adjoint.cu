// Placeholder: replaced by the checkpointed adjoint.
#include "pg_system.cuh"
struct pg_adjoint {};
size_t pg_system::adjoint_bytes() const { return 0; }
namespace pg {
void destroy_adjoint(pg_system* s) { delete s->adj; s->adj = nullptr; }
}
extern "C" {
int pg_forward_checkpointed(pg_system*, int, int) { pg::set_error("not built"); return PG_ESTATE; }
int pg_backward(pg_system*, const double*, double*, double*, double*) { pg::set_error("not built"); return PG_ESTATE; }
int pg_autotune(pg_system*, int, int*, double*, int*, double*) { pg::set_error("not built"); return PG_ESTATE; }
}
