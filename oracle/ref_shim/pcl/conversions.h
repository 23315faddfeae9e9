// Host stand-in (TEST INFRASTRUCTURE ONLY): ros_tsdf includes this header but
// uses nothing from it on the integration path.
#pragma once
#include "point_types.h"
