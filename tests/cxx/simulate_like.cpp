// Compile check: the drop-in classes instantiate against libvvhd's own Space/TBody/TObj
// and are used exactly the way utils/vvflow/vvflow.cpp:200-255 uses the reference classes.
#include "TSpace.hpp"
#include "vvgpu_modules.hpp"

#include <limits>

using TSortedTree = vvgpu_cxx::stree<Space>;
using MConvectiveFast = vvgpu_cxx::MConvectiveFast<Space>;
using MEpsilonFast = vvgpu_cxx::MEpsilonFast<Space>;
using MDiffusiveFast = vvgpu_cxx::MDiffusiveFast<Space>;

int one_step(Space& S) {
    bool is_viscous = (S.re != std::numeric_limits<double>::infinity());
    double dl = S.average_segment_length();
    double min_node_size = dl > 0 ? dl * 5 : 0;
    double max_node_size = dl > 0 ? dl * 100 : std::numeric_limits<double>::max();
    TSortedTree tr = {&S, 8, min_node_size, max_node_size};
    MConvectiveFast convective = {&S, &tr};
    MEpsilonFast epsilon = {&S, &tr};
    MDiffusiveFast diffusive = {&S, &tr};
    const void* collision = nullptr;
    if (S.BodyList.size()) {
        tr.build();
        convective.calc_circulation(&collision);
        tr.destroy();
    }
    tr.build();
    epsilon.CalcEpsilonFast(is_viscous);
    convective.process_all_lists();
    TVec v = convective.velocity(TVec(1, 2));
    if (is_viscous) {
        diffusive.process_vort_list();
        diffusive.process_heat_list();
    }
    const auto& bn = tr.getBottomNodes();
    const auto* node = tr.findNode(TVec(0.5, 0.5));
    int n = (int)bn.size() + (node ? (int)node->vRange.size() : 0) + epsilon.Merged() + (v.x > 0);
    tr.printBottomNodes(stderr, false);
    tr.destroy();
    return n;
}
