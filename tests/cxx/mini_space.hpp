// A minimal host Space with the members the drop-in classes of include/vvgpu_modules.hpp
// read and write, laid out like libvvhd's (TObj.hpp:10-35, TBody.hpp:17-158,
// TSpace.hpp:19-129): the vortex list as a vector of TObj, bodies as shared pointers with a
// list of TAtt segments (a TAtt is a TObj).  Test infrastructure for running the drop-in
// where the reference's own classes are not built.
#pragma once

#include <cmath>
#include <cstdint>
#include <limits>
#include <memory>
#include <vector>

namespace mini {

struct TVec {
    double x = 0, y = 0;
    TVec() = default;
    TVec(double a, double b) : x(a), y(b) {}
};

struct TVec3D {
    TVec r;
    double o = 0;
};

struct TObj {
    TVec r;
    double g = 0;
    TVec v;
    double _1_eps = 0;
};

struct TAtt : TObj {
    TVec corner;
    double gsum = 0, fric = 0, Cp = 0, Fr = 0, Nu = 0;
    uint32_t slip = 0;
};

struct TBody {
    enum class bc_t { steady, kutta };
    std::vector<TAtt> alist;
    TVec3D holder, dpos, speed_slae, speed_slae_prev, friction_prev, fdt_dead, force_hydro, force_holder;
    TVec3D kspring;
    double g_dead = 0, density = 1;
    int32_t special_segment_no = 0;
    bc_t boundary_condition = bc_t::steady;
    TBody() {
        const double inf = std::numeric_limits<double>::infinity();
        kspring.r = TVec(inf, inf);
        kspring.o = inf;
    }
    TVec3D speed(double) const { return TVec3D{}; }  // a body at rest
};

struct Space {
    std::vector<TObj> VortexList;
    std::vector<TObj> HeatList;
    std::vector<std::shared_ptr<TBody>> BodyList;
    double re = 600, dt = 0.005, time = 0, inf_g = 0;
    TVec inf_vel{1, 0}, gravity{0, 0};
    TVec inf_speed() const { return inf_vel; }
    // Space::average_segment_length (TSpace.hpp:119-129): the first body's perimeter over
    // its segment count minus one
    double average_segment_length() const {
        if (BodyList.empty() || BodyList[0]->alist.size() < 2) return std::numeric_limits<double>::infinity();
        const auto& a = BodyList[0]->alist;
        double slen = 0;
        for (size_t k = 0; k < a.size(); k++) {
            const TVec& p = a[k].corner;
            const TVec& q = a[(k + 1) % a.size()].corner;
            slen += std::sqrt((q.x - p.x) * (q.x - p.x) + (q.y - p.y) * (q.y - p.y));
        }
        return slen / (double)(a.size() - 1);
    }
};

}  // namespace mini
