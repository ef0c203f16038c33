// ytgb_internal.h -- declarations shared between the host and CUDA halves of
// libytgb (not part of the public C ABI).
#pragma once
#include <string>

void ytgb_set_error(const std::string &msg);

// device error codes written to the caller's error word
#define YTGB_DEVERR_STEP_LIMIT 1      // a DDA walk exceeded its step bound
#define YTGB_DEVERR_BAD_BRICK 2       // brick index / dims out of range
#define YTGB_DEVERR_BAD_TF 3          // transfer function header inconsistent
#define YTGB_DEVERR_BAD_CELL 4        // an off-axis cell's stamp level out of range

// FNV-1a 64-bit offset basis and prime (traversal trace)
#define YTGB_FNV_OFFSET 1469598103934665603ull
#define YTGB_FNV_PRIME 1099511628211ull
