// Project-written stand-in for the Space constructor of libvvhd/src/TSpace.cpp, whose
// translation unit needs HDF5 (absent here). TEST INFRASTRUCTURE ONLY.
// Field defaults follow TSpace.cpp:14-36.
#include "TSpace.hpp"

#include <limits>

static const double shim_inf = std::numeric_limits<double>::infinity();

Space::Space()
    : caption(), re(shim_inf), pr(0), inf_g(), inf_vx(), inf_vy(), inf_marker(), gravity(),
      time(), dt(1, 1), dt_save(), dt_streak(), dt_profile(), finish(shim_inf), BodyList(),
      VortexList(), HeatList(), SourceList(), StreakSourceList(), StreakList() {}
