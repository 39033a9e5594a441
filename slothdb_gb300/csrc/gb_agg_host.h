// gb_agg_host.h — host-side hooks shared between translation units.
#pragma once
#include "../../include/slothdb_gb300.h"

// Applies default (or autotuned) launch parameters to a freshly compiled
// handle: shared-table slots, CTAs per SM, block size.
void gb_apply_tuning(gb_agg *h);
