// The C-ABI simulation handle (opaque to callers; include/cipc.h declares it).
#pragma once
#include "../../include/cipc.h"
#include "cipc_util.h"
#include "sim.h"

struct cipc_sim {
    cipc::Sim* s;
};

static inline int check_sim(cipc_sim* h)
{
    if (!h || !h->s) return cipc::set_error(CIPC_ERR_INVALID_ARG, "null simulation handle");
    return CIPC_OK;
}
