// Project-written stand-in for libvvhd/src/TEval.cpp (which embeds Lua 5.2, absent here).
// TEST INFRASTRUCTURE ONLY: lets the reference's own hot-path sources link unmodified.
// Expressions are restricted to numeric constants; eval() keeps the reference's
// `#pragma omp critical` around the cached lookup (TEval.cpp:165-204) so the timed CPU
// baseline pays the same serialisation per call as the reference does.
#include "TEval.hpp"

#include <cmath>
#include <cstdlib>
#include <limits>
#include <stdexcept>

static const double shim_nan = std::numeric_limits<double>::quiet_NaN();

TEval::TEval()
    : lua_state(nullptr), expr(), cacheTime1(shim_nan), cacheTime2(shim_nan),
      cacheValue1(), cacheValue2() {}

TEval::~TEval() {}

TEval::TEval(const TEval& copy) : TEval() { *this = std::string(copy); }

TEval::TEval(const std::string& str) : TEval() { *this = str; }

TEval& TEval::operator=(const TEval& copy) { return *this = std::string(copy); }

TEval& TEval::operator=(const std::string& str) {
    if (str.empty()) {
        expr.clear();
        return *this;
    }
    char* end = nullptr;
    double v = std::strtod(str.c_str(), &end);
    if (end == str.c_str()) throw std::invalid_argument("TEval shim: constant expected");
    expr = str;
    cacheTime1 = cacheTime2 = shim_nan;
    cacheValue1 = cacheValue2 = v;
    return *this;
}

double TEval::eval(double t) const {
    if (expr.empty()) return 0;
    double ret = 0;
#pragma omp critical
    {
        if (t == cacheTime1) {
            ret = cacheValue1;
        } else {
            ret = std::strtod(expr.c_str(), nullptr);
            cacheTime2 = cacheTime1;
            cacheValue2 = cacheValue1;
            cacheTime1 = t;
            cacheValue1 = ret;
        }
    }
    return ret;
}
