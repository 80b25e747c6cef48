// report.cpp -- the reference's headless Report programs, on the drop-in classes.
//
//   report xfront  [dir]     DamBreak.Report/XFrontTest.h:16-90   -> XFrontOutput
//   report yfront  [dir]     DamBreak.Report/YFrontTest.h:16-94   -> YFrontOutput
//   report poiseuille [dir]  Poiseuille.Report/dump.h:15-86      -> XVelocityYPosition<t>.dat
//   report density [dir] [T] Peristalsis.Report/density.h:12-70  -> density.dat
//   report forces  [dir] [T] Peristalsis.Report/forces.h:13-88   -> press_{x,y}.dat, visc_{x,y}.dat
//   report velocityfield [dir]  Peristalsis.Report/velocityfield.h:16-91
//                                                 -> velocity_field0x3.dat, velocity_field0x4.dat
//   report pvprofile [dir]   Peristalsis.Report/poiseuille_velocity_profile.h:13-94
//                                                 -> velocity_profile<t>.dat
//   report pvprofile_noslip [dir]  the same with no-slip moving-wall extrapolation
//
// Same scenes, time frames and output formats as the reference.  The front,
// height and per-step averages come from device reductions over the fluid
// particles instead of copying every particle to the host and sorting there.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cmag/systems.hpp>

namespace {

std::string path(const std::string &dir, const std::string &name) { return dir + "/" + name; }

// XFrontTest.h:45-62 (dimensionless time, surge front), Martin & Moyce table 2
const float kXFront[][2] = {{0.00f, 1.0f},  {0.41f, 1.11f}, {0.84f, 1.22f}, {1.19f, 1.44f},
                            {1.43f, 1.67f}, {1.63f, 1.89f}, {1.83f, 2.11f}, {1.98f, 2.33f},
                            {2.20f, 2.56f}, {2.32f, 2.78f}, {2.51f, 3.00f}, {2.65f, 3.22f},
                            {2.83f, 3.44f}, {2.97f, 3.67f}, {3.11f, 3.89f}};
// YFrontTest.h:136-153 (dimensionless time, column height), table 6
const float kYFront[][2] = {{0.0f, 1.0f},   {0.56f, 0.94f}, {0.77f, 0.89f}, {0.93f, 0.83f},
                            {1.08f, 0.78f}, {1.28f, 0.72f}, {1.46f, 0.67f}, {1.66f, 0.61f},
                            {1.84f, 0.56f}, {2.00f, 0.50f}, {2.21f, 0.44f}, {2.45f, 0.39f},
                            {2.70f, 0.33f}, {3.06f, 0.28f}, {3.44f, 0.22f}};

DamBreakSystem *relaxed_column()
{
    const int num = 128;
    const float radius = 1.0f / (2 * num);
    DamBreakSystem *s = new DamBreakSystem(make_uint3(num, 2 * num, 1), 1, make_uint3(512, 256, 4),
                                           radius, false);
    s->reset();
    while (s->getElapsedTime() < 1.5f) s->update();  // relax
    std::printf("relaxed at t = %f\n", s->getElapsedTime());
    s->removeRightBoundary();
    return s;
}

int xfront(const std::string &dir)
{
    const int num = 128, off = 1;
    const float radius = 1.0f / (2 * num);
    DamBreakSystem *s = relaxed_column();
    const float xwidth = (num + off) * 2 * radius;
    const float scale = std::sqrt(2 * std::fabs(s->getGravity().y) / xwidth);
    FILE *f = std::fopen(path(dir, "XFrontOutput").c_str(), "w");
    for (const auto &fr : kXFront) {
        while (s->getElapsedTime() * scale < fr[0]) s->update();
        const float x = s->fluidMax().x;
        std::fprintf(f, "%f %f %f %f \n", fr[0], s->getElapsedTime(), fr[1],
                     (x + radius - s->getWorldOrigin().x) / xwidth);
    }
    std::fclose(f);
    delete s;
    return 0;
}

int yfront(const std::string &dir)
{
    const int num = 128;
    const float radius = 1.0f / (2 * num);
    DamBreakSystem *s = relaxed_column();
    const float yheight = s->fluidMax().y + radius - s->getWorldOrigin().y;
    const float scale = std::sqrt(2 * std::fabs(s->getGravity().y) / yheight);
    FILE *f = std::fopen(path(dir, "YFrontOutput").c_str(), "w");
    for (const auto &fr : kYFront) {
        while (s->getElapsedTime() * scale < fr[0]) s->update();
        const float y = s->fluidMax().y;
        std::fprintf(f, "%f %f %f %f \n", fr[0], s->getElapsedTime(), fr[1],
                     (y + radius - s->getWorldOrigin().y) / yheight);
    }
    std::fclose(f);
    delete s;
    return 0;
}

int poiseuille(const std::string &dir)
{
    const int off = 3;
    const uint3 grid = make_uint3(16, 64, 4);
    const float radius = 1.0f / (2 * (grid.y - 2 * off) * 1000);
    PoiseuilleFlowSystem s(make_uint3(grid.x, grid.y - 2 * off, 1), off, grid, radius, false);
    s.reset();
    const int n = s.getNumParticles();
    std::vector<float> pos(4 * (size_t)n), vel(4 * (size_t)n);
    const float frames[] = {0.0225f, 0.045f, 0.1125f, 0.225f, 1.0f};
    for (float t : frames) {
        while (s.getElapsedTime() < t) s.update();
        s.getArray(CMAG_POSITION, pos.data(), 0, n);
        s.getArray(CMAG_VELOCITY, vel.data(), 0, n);
        char name[64];
        std::snprintf(name, sizeof(name), "XVelocityYPosition%g.dat", t);
        FILE *f = std::fopen(path(dir, name).c_str(), "w");
        std::fprintf(f, "0.0 0.0\n");
        for (int i = 0; i < n; ++i) {
            const float *p = &pos[4 * (size_t)i];
            if (p[0] > 0 && p[0] < 2 * radius && p[3] == 0.0f)
                std::fprintf(f, "%g %g\n", vel[4 * (size_t)i],
                             p[1] + std::fabs(s.getWorldOrigin().y) - off * 2 * radius);
        }
        std::fprintf(f, "0.000000 0.001000\n");
        std::fclose(f);
    }
    return 0;
}

PeristalsisSystem *channel()
{
    const int off = 3;
    const float c = std::pow(10.0f, -4.0f);
    const float radius = 1.0f / (2 * (64 - 6) * 1000);
    return new PeristalsisSystem(std::pow(10.0f, -4.0f), make_uint3(256, 64 - 2 * off, 1),
                                 0.6f * 35 * radius, 100 * c, c, make_float3(0, 0, 0), off,
                                 make_uint3(256, 128, 4), radius, false);
}

int density(const std::string &dir, float until)
{
    PeristalsisSystem *s = channel();
    s->Reset();
    const uint32_t fluid = 256 * 58;
    FILE *f = std::fopen(path(dir, "density.dat").c_str(), "w");
    while (s->GetElapsedTime() < until) {
        s->Update();
        std::fprintf(f, "%g %g\n", s->GetElapsedTime(), s->fluidAverage(CMAG_MEASURES, fluid).x);
    }
    std::fclose(f);
    delete s;
    return 0;
}

int forces(const std::string &dir, float until)
{
    PeristalsisSystem *s = channel();
    s->Reset();
    const uint32_t fluid = 256 * 58;
    const char *names[4] = {"press_x.dat", "press_y.dat", "visc_x.dat", "visc_y.dat"};
    FILE *f[4];
    for (int k = 0; k < 4; ++k) f[k] = std::fopen(path(dir, names[k]).c_str(), "w");
    while (s->GetElapsedTime() < until) {
        s->Update();
        const float4 pr = s->fluidAverage(CMAG_PRESSUREFORCE, fluid);
        const float4 vi = s->fluidAverage(CMAG_VISCOUSFORCE, fluid);
        const float t = s->GetElapsedTime();
        std::fprintf(f[0], "%g %g\n", t, pr.x);
        std::fprintf(f[1], "%g %g\n", t, pr.y);
        std::fprintf(f[2], "%g %g\n", t, vi.x);
        std::fprintf(f[3], "%g %g\n", t, vi.y);
    }
    for (int k = 0; k < 4; ++k) std::fclose(f[k]);
    delete s;
    return 0;
}

// the reference's file-name rule: ostream << t, then character 1 replaced by "x"
// (appended when the number has a single character): 0.3 -> 0x3, 1 -> 1x
std::string frame_name(const char *stem, float t)
{
    char num[32];
    std::snprintf(num, sizeof(num), "%g", t);
    std::string s(num);
    s.replace(1, 1, "x");
    return std::string(stem) + s + ".dat";
}

// every fourth particle's position and velocity at t = 0.3 and 0.4 s
int velocityfield(const std::string &dir)
{
    PeristalsisSystem *s = channel();
    s->Reset();
    const int n = s->getNumParticles();
    std::vector<float> pos(4 * (size_t)n), vel(4 * (size_t)n);
    for (float t : {0.3f, 0.4f}) {
        while (s->GetElapsedTime() < t) s->Update();
        s->getArray(CMAG_POSITION, pos.data(), 0, n);
        s->getArray(CMAG_VELOCITY, vel.data(), 0, n);
        FILE *f = std::fopen(path(dir, frame_name("velocity_field", t)).c_str(), "w");
        for (int i = 0; i < n; i += 4)
            std::fprintf(f, "%g %g %g %g\n", pos[4 * (size_t)i], pos[4 * (size_t)i + 1],
                         vel[4 * (size_t)i], vel[4 * (size_t)i + 1]);
        std::fclose(f);
    }
    delete s;
    return 0;
}

// The Peristalsis solver as a plain channel (amplitude 0, body force 1e-4):
// leap-frog u_x against height in the first column of cells, in sorted order.
// noslip: with the no-slip extrapolation into the walls (an option of this
// build; the reference keeps it commented out).
int pvprofile(const std::string &dir, bool noslip)
{
    const int off = 3, sizex = 64;
    const float c = std::pow(10.0f, -4.0f);
    const float radius = 1.0f / (2 * (sizex - 2 * off) * 1000);
    const uint3 grid = make_uint3(sizex, 64, 4);
    const uint3 fluid = make_uint3(grid.x, grid.y - 2 * off, 1);
    PeristalsisSystem *s = new PeristalsisSystem(std::pow(10.0f, -4.0f), fluid, 0, 0, c,
                                                 make_float3(std::pow(10.0f, -4.0f), 0, 0), off,
                                                 grid, radius, false);
    if (noslip) {
        cmag_sph_params p = s->params();
        p.wall_noslip = 1;
        s->setParams(p);
    }
    s->Reset();
    const int n = s->getNumParticles();
    std::vector<float> pos(4 * (size_t)n), vlf(4 * (size_t)n);
    std::vector<uint32_t> index(n);
    for (float t : {0.0225f, 0.045f, 0.1125f, 0.225f, 1.0f}) {
        while (s->GetElapsedTime() < t) s->Update();
        s->getArray(CMAG_POSITION, pos.data(), 0, n);
        s->getArray(CMAG_VELOCITYLEAPFROG, vlf.data(), 0, n);
        cmag::check(cmag_system_get_uint_array(s->handle(), CMAG_INDEX, index.data(), 0, n), s->handle());
        const float bottom = s->getWorldOrigin().y + 2 * s->getradius() * off;
        FILE *f = std::fopen(path(dir, frame_name("velocity_profile", t)).c_str(), "w");
        std::fprintf(f, "0 0\n");
        for (int i = 0; i < n; ++i) {
            const float *p = &pos[4 * (size_t)index[i]];
            if (p[0] > 0 && p[0] < 2 * s->getradius() && p[1] > bottom &&
                p[1] < bottom + fluid.y * 2.0f * radius)
                std::fprintf(f, "%g %g\n", vlf[4 * (size_t)index[i]],
                             p[1] - s->getWorldOrigin().y - off * 2 * s->getradius());
        }
        std::fprintf(f, "0 0.001\n");
        std::fclose(f);
    }
    delete s;
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: report xfront|yfront|poiseuille|density|forces|velocityfield|pvprofile|pvprofile_noslip [dir] [until]\n");
        return 2;
    }
    const std::string what = argv[1], dir = argc > 2 ? argv[2] : ".";
    const float until = argc > 3 ? (float)std::atof(argv[3]) : 1.0f;
    try {
        if (what == "xfront") return xfront(dir);
        if (what == "yfront") return yfront(dir);
        if (what == "poiseuille") return poiseuille(dir);
        if (what == "density") return density(dir, until);
        if (what == "forces") return forces(dir, until);
        if (what == "velocityfield") return velocityfield(dir);
        if (what == "pvprofile") return pvprofile(dir, false);
        if (what == "pvprofile_noslip") return pvprofile(dir, true);
    } catch (const cmag::Error &e) {
        std::fprintf(stderr, "cmag error %d: %s\n", e.code, e.what());
        return 1;
    }
    std::fprintf(stderr, "unknown report %s\n", what.c_str());
    return 2;
}
