// One step of the hot path driven through the C++ drop-in classes exactly as
// utils/vvflow/vvflow.cpp:200-255 drives the reference's (tree build, calc_circulation, tree
// destroy, tree build, CalcEpsilonFast, process_all_lists, process_vort_list, a velocity(p)
// probe, tree destroy), on a mini::Space read from a file; the Space is written back after
// the step.  Test infrastructure (tests/test_gpu_dropin.py).
//
//   dropin_step <in.bin> <out.bin>
// in:  int64 n, m; double re, dt, inf_x, inf_y, far_criteria, probe_x, probe_y;
//      n x (x, y, g, _1_eps); m x (corner x, corner y)
// out: int64 n, m, merged; n x (x, y, g, _1_eps, vx, vy); m x (g, fric);
//      9 x body unknowns (speed_slae, force_hydro, force_holder); probe vx, vy
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "mini_space.hpp"
#include "vvgpu_modules.hpp"

using Space = mini::Space;
using TSortedTree = vvgpu_cxx::stree<Space>;
using MConvectiveFast = vvgpu_cxx::MConvectiveFast<Space>;
using MEpsilonFast = vvgpu_cxx::MEpsilonFast<Space>;
using MDiffusiveFast = vvgpu_cxx::MDiffusiveFast<Space>;

template <class T>
static void rd(FILE* f, T* p, size_t n) {
    if (fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short input");
}
template <class T>
static void wr(FILE* f, const T* p, size_t n) {
    if (fwrite(p, sizeof(T), n, f) != n) throw std::runtime_error("short write");
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    try {
        FILE* in = fopen(argv[1], "rb");
        if (!in) return 3;
        int64_t nm[2];
        double prm[7];
        rd(in, nm, 2);
        rd(in, prm, 7);
        Space S;
        S.re = prm[0];
        S.dt = prm[1];
        S.inf_vel = mini::TVec(prm[2], prm[3]);
        S.VortexList.resize(nm[0]);
        for (auto& o : S.VortexList) {
            double r[4];
            rd(in, r, 4);
            o.r = mini::TVec(r[0], r[1]);
            o.g = r[2];
            o._1_eps = r[3];
        }
        if (nm[1] > 0) {
            auto b = std::make_shared<mini::TBody>();
            b->alist.resize(nm[1]);
            for (auto& a : b->alist) {
                double c[2];
                rd(in, c, 2);
                a.corner = mini::TVec(c[0], c[1]);
            }
            S.BodyList.push_back(b);
        }
        fclose(in);

        // simulate() (utils/vvflow/vvflow.cpp:200-255), without the shed and the move
        const double dl = S.average_segment_length();
        const double min_node = dl > 0 && dl < 1e300 ? dl * 5 : 0;
        const double max_node = dl > 0 && dl < 1e300 ? dl * 100 : std::numeric_limits<double>::max();
        TSortedTree tr(&S, prm[4], min_node, max_node, VVGPU_FP64, 0);
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
        epsilon.CalcEpsilonFast(true);
        convective.process_all_lists();
        diffusive.process_vort_list();
        const mini::TVec pv = convective.velocity(mini::TVec(prm[5], prm[6]));
        tr.destroy();

        FILE* out = fopen(argv[2], "wb");
        if (!out) return 4;
        const int64_t hdr[3] = {(int64_t)S.VortexList.size(), nm[1], (int64_t)epsilon.Merged()};
        wr(out, hdr, 3);
        for (auto& o : S.VortexList) {
            const double r[6] = {o.r.x, o.r.y, o.g, o._1_eps, o.v.x, o.v.y};
            wr(out, r, 6);
        }
        for (auto& b : S.BodyList)
            for (auto& a : b->alist) {
                const double r[2] = {a.g, a.fric};
                wr(out, r, 2);
            }
        double u[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (!S.BodyList.empty()) {
            const auto& b = *S.BodyList[0];
            const double t[9] = {b.speed_slae.r.x, b.speed_slae.r.y, b.speed_slae.o, b.force_hydro.r.x,
                                 b.force_hydro.r.y, b.force_hydro.o, b.force_holder.r.x, b.force_holder.r.y,
                                 b.force_holder.o};
            for (int k = 0; k < 9; k++) u[k] = t[k];
        }
        wr(out, u, 9);
        const double p[2] = {pv.x, pv.y};
        wr(out, p, 2);
        fclose(out);
    } catch (std::exception& e) {
        fprintf(stderr, "dropin_step: %s\n", e.what());
        return 1;
    }
    return 0;
}
