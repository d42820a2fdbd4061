// gbsph_motion_internal.h -- what the context needs to know of a motion.
#pragma once
#include "gbsph.h"

namespace gbmotion {
unsigned object_count(const gbsph_motion* m);
const gbsph_motion_object* objects(const gbsph_motion* m);
}  // namespace gbmotion
