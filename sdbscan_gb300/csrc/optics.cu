// sOPTICS stage: placeholder until the neighbour-list and ordering kernels land.
#include "common.cuh"
#include "engine_internal.h"

sdb_status sdb_engine::optics_stage(float, int, int&) {
    return fail(SDB_ERR_INTERNAL, "sOPTICS is not implemented yet");
}
