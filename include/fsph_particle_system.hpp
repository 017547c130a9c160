/*
 * fsph_particle_system.hpp -- C++ drop-in for the reference's particle-system
 * classes, over the C ABI of fsph.h (header only; link libfsph.so).
 *
 * Same class, type and method names as rxParticleSystemBase (rx_ps.h:55-333),
 * rxSPH (rx_sph.h:202-426) and rxPBDSPH (rx_sph.h:1027-1274), with the same
 * argument meaning and error behaviour, so that a caller written against
 * rx_ps.h (e.g. the InitSPH / StepPS sequence, rx_fltk_glcanvas.cpp:2386-2496)
 * compiles against this header:
 *   - construction is two-phase, `new rxPBDSPH(use_opengl)` then
 *     Initialize(const rxSPHEnviroment&) (rx_sph_pbd.cpp:102-201), which
 *     derives h, r and rho0 from the environment as the reference does;
 *     the GPU context is created there.  A constructor taking fsph_params
 *     (explicit h / rho0 / m) is there too;
 *   - Update returns false when there is nothing to step (N = 0), as
 *     rxPBDSPH_GPU::Update does (rx_sph_pbd_gpu.cpp:818);
 *   - UpdateWithoutPosAndVel evaluates a step's fields without moving the
 *     particles (rxSPH_GPU::UpdateWithoutPosAndVel, rx_sph_gpu.cpp:925);
 *   - GetArrayVBO returns a NON-OWNING pointer to an internal host buffer,
 *     refreshed from the device when d2h is true (rx_sph_pbd_gpu.cpp:2497-2613),
 *     vectors with the DIM = 4 stride;
 *   - GetParticleDevice returns a borrowed device pointer (device order; the
 *     reference's CPU class returned a fresh copy the caller freed,
 *     rx_sph_pbd.cpp:499-509);
 *   - SetParticlesToCell() / SetParticlesToCell(prts, n, h) fill the
 *     neighbour lists that GetNeights() returns as vector<vector<rxNeigh>>
 *     (rx_sph_pbd.cpp:1735-1750, rx_nnsearch.h:59-64): Idx and Dist2 as the
 *     reference fills them (squared distance in double, rounded to float),
 *     and Dist = sqrt(Dist2), which the reference leaves unset;
 *   - AddBox / AddSphere / Reset place particles as rx_ps.cpp:66-261 do, with
 *     the jitter drawn from a seeded counter-based generator instead of
 *     srand(time(NULL)), so a scene is reproducible;
 *   - Vec3 arguments accept any type with operator[] (the reference's Vec3
 *     included); this header's Vec3 is a minimal stand-in.
 * The status of the last failing call is LastStatus() / LastError().
 * GL-only members (SetColorVBO, Draw*, VBO ids) do not exist here.
 */
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "fsph.h"

namespace fsph_gb300 {

typedef float RXREAL;
typedef unsigned int uint;

/* Three doubles with the vector operations the operator surface needs. */
struct Vec3 {
    double data[3];
    Vec3() : data{0.0, 0.0, 0.0} {}
    Vec3(double a) : data{a, a, a} {}  // NOLINT: as the reference's Vec3(0.0)
    Vec3(double x, double y, double z) : data{x, y, z} {}
    template <class V, class = decltype(std::declval<const V &>()[2]),
              class = typename std::enable_if<!std::is_arithmetic<V>::value>::type>
    Vec3(const V &v) : data{(double)v[0], (double)v[1], (double)v[2]} {}  // NOLINT: any indexable vector
    double &operator[](int i) { return data[i]; }
    double operator[](int i) const { return data[i]; }
    Vec3 operator+(const Vec3 &b) const { return Vec3(data[0] + b[0], data[1] + b[1], data[2] + b[2]); }
    Vec3 operator-(const Vec3 &b) const { return Vec3(data[0] - b[0], data[1] - b[1], data[2] - b[2]); }
    Vec3 operator*(double s) const { return Vec3(s * data[0], s * data[1], s * data[2]); }
    Vec3 operator/(double s) const { return Vec3(data[0] / s, data[1] / s, data[2] / s); }
    Vec3 &operator+=(const Vec3 &b) { for (int k = 0; k < 3; ++k) data[k] += b[k]; return *this; }
    Vec3 &operator-=(const Vec3 &b) { for (int k = 0; k < 3; ++k) data[k] -= b[k]; return *this; }
};
inline Vec3 operator*(double s, const Vec3 &a) { return a * s; }

/* Inlet line (rx_ps.h:41-49). */
struct rxInletLine {
    Vec3 pos1, pos2;  /* end points */
    Vec3 vel;         /* velocity of the added particles */
    Vec3 up;          /* direction the rows pile up in */
    int accum;        /* rows per emission */
    int span;         /* steps between emissions */
    double spacing;   /* row spacing, in particle spacings */
};

/* Neighbour record (rx_nnsearch.h:59-64). */
struct rxNeigh {
    int Idx;
    RXREAL Dist;
    RXREAL Dist2;
};

/* Scene parameters (rx_sph.h:95-182), the reference's defaults. */
struct rxSPHEnviroment {
    enum { MAX_DELETE_REGIONS = 64 };
    int max_particles = 50000;
    Vec3 boundary_cen = Vec3(0.0);
    Vec3 boundary_ext = Vec3(2.0, 0.8, 0.8);
    RXREAL dens = (RXREAL)998.29;
    RXREAL mass = (RXREAL)0.04;
    RXREAL kernel_particles = (RXREAL)20.0;
    RXREAL dt = (RXREAL)0.01;
    RXREAL viscosity = (RXREAL)1.0e-3;
    RXREAL gas_k = (RXREAL)3.0;
    int use_inlet = 0;
    RXREAL et_cri = (RXREAL)1.0;
    RXREAL epsilon = (RXREAL)0.001;
    RXREAL eta = (RXREAL)0.05;
    int min_iter = 2;
    int max_iter = 10;
    int use_ap = 1;
    RXREAL ap_k = (RXREAL)0.1;
    RXREAL ap_n = (RXREAL)4.0;
    RXREAL ap_q = (RXREAL)0.2;
    int use_delete_region = 0;
    Vec3 delete_region[MAX_DELETE_REGIONS][2];
    Vec3 mesh_boundary_cen = Vec3(0.0);
    Vec3 mesh_boundary_ext = Vec3(0.0);
    int mesh_vertex_store = 10;
    int mesh_max_n = 128;
};

namespace detail {
/* U[0, 1) from (seed, index): SplitMix64 finaliser (Steele, Lea, Flood 2014) */
inline double uniform01(uint64_t seed, uint64_t idx) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + idx * 0xD1B54A32D192ED03ull + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
}  // namespace detail

/* rxParticleSystemBase over one fsph context: the reference's non-virtual
 * members (the state, the settings, scene set-up, file I/O) and its pure
 * virtuals, which rxFsphSolver implements for both solvers. */
class rxParticleSystemBase {
public:
    enum rxParticleConfig { RX_CONFIG_RANDOM, RX_CONFIG_GRID, RX_CONFIG_BOX, RX_CONFIG_NONE, _NUM_CONFIGS };
    /* rx_ps.h:68-116; the arrays this library holds are the ones the fluid
     * step produces (the others return nullptr from GetArrayVBO) */
    enum rxParticleArray {
        RX_POSITION = 0, RX_VELOCITY, RX_NORMAL, RX_FORCE, RX_DENSITY, RX_PRESSURE,
        RX_SURFACE, RX_ATTRIBUTE,
        RX_PREDICT_POS, RX_PREDICT_VEL, RX_SCALING_FACTOR, RX_CORRECTION,
        RX_BOUNDARY_PARTICLE, RX_BOUNDARY_PARTICLE_VOL,
        RX_TEST, RX_DEBUG_VECTOR,
        RX_TURB_VELOCITY, RX_ENERGY_SPECTRUM, RX_VORTICITY,
        RX_UPDATED_POSITION, RX_EIGEN_VALUE, RX_ROTATION_MATRIX, RX_TRANSFORMATION, RX_SUBPOSITION,
        RX_CONSTANT, RX_RAMP, RX_NONE,
        RX_TEMP, RX_SHPMTCHNG, RX_ICE_CONNECT, RX_ICE_CALC, RX_EDGE, RX_ICE_FAST_PATH, RX_ICE_SELECTED,
        RX_ICE_DEFORMATION,
        RX_PSDATA_END
    };

    explicit rxParticleSystemBase(int solver, bool use_opengl = false) : m_solver(solver) { (void)use_opengl; }
    rxParticleSystemBase(const fsph_params &p, int solver) : m_solver(solver) { create(p); }
    virtual ~rxParticleSystemBase() {
        if (m_ctx) fsph_destroy(m_ctx);
    }
    rxParticleSystemBase(const rxParticleSystemBase &) = delete;
    rxParticleSystemBase &operator=(const rxParticleSystemBase &) = delete;

    /* pure virtuals of rx_ps.h:253-275 (SetColorVBO, a GL call, excepted) */
    virtual bool Update(RXREAL dt, int step = 0) = 0;
    virtual bool UpdateWithoutPosAndVel(RXREAL dt, int step = 0) = 0;
    virtual RXREAL *GetArrayVBO(rxParticleArray type, bool d2h = true, int num = -1) = 0;
    virtual void SetArrayVBO(rxParticleArray type, const RXREAL *data, int start, int count) = 0;
    virtual void SetArrayVBO(rxParticleArray type, const int *data, int start, int count) = 0;
    virtual RXREAL *GetParticle(void) = 0;
    virtual RXREAL *GetParticleDevice(void) = 0;
    virtual void SetParticlesToCell(void) = 0;
    virtual void SetParticlesToCell(RXREAL *prts, int n, RXREAL h) = 0;


    /* Initialize(env) (rx_sph_pbd.cpp:102-201, rx_sph_cpu.cpp:92-166): h, r
     * and rho0 derived from the environment; returns on failure with
     * LastStatus() set */
    void Initialize(const rxSPHEnviroment &env) {
        fsph_env e;
        std::memset(&e, 0, sizeof(e));
        e.solver = m_solver;
        e.max_particles = env.max_particles;
        for (int k = 0; k < 3; ++k) {
            e.boundary_cen[k] = env.boundary_cen[k];
            e.boundary_ext[k] = env.boundary_ext[k];
        }
        e.dens = env.dens; e.mass = env.mass; e.kernel_particles = env.kernel_particles;
        e.viscosity = env.viscosity; e.gas_k = env.gas_k;
        e.epsilon = env.epsilon; e.eta = env.eta; e.min_iter = env.min_iter; e.max_iter = env.max_iter;
        e.use_ap = env.use_ap; e.ap_k = env.ap_k; e.ap_n = env.ap_n; e.ap_q = env.ap_q;
        e.gravity_y = -9.82f; /* rxParticleSystemBase constructor (rx_ps.h:165) */
        fsph_params p;
        m_status = fsph_params_from_env(&e, &p);
        if (m_status != FSPH_OK) return;
        p.gravity[1] = m_gravity_y;
        create(p);
        /* the deletion regions of the environment (rx_sph_pbd_gpu.cpp:264-271) */
        for (int i = 0; m_ctx && i < env.use_delete_region && i < rxSPHEnviroment::MAX_DELETE_REGIONS; ++i)
            fsph_add_delete_region(m_ctx, env.delete_region[i][0].data, env.delete_region[i][1].data);
    }

    bool IsInitialized() const { return m_ctx != nullptr; }
    int LastStatus() const { return m_status; }
    std::string LastError() const { return m_ctx ? fsph_last_error(m_ctx) : fsph_status_string(m_status); }

    /* -- particle data -------------------------------------------------- */
    /* Set(ppos, pvel) (rx_ps.cpp:30-59): the sizes must agree; any vector
     * type with operator[] (Vec3 or the reference's Vec3) */
    template <class V, class = decltype(std::declval<const V &>()[2])>
    bool Set(const std::vector<V> &ppos, const std::vector<V> &pvel) {
        if (ppos.empty() || ppos.size() != pvel.size()) return false;
        const int n = (int)ppos.size();
        std::vector<float> p4(4 * (size_t)n, 0.0f), v4(4 * (size_t)n, 0.0f);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                p4[4 * (size_t)i + k] = (float)ppos[i][k];
                v4[4 * (size_t)i + k] = (float)pvel[i][k];
            }
        return set4(p4, v4, n);
    }
    /* the same from xyz triples */
    bool Set(const std::vector<float> &pos3, const std::vector<float> &vel3) {
        if (pos3.empty() || pos3.size() % 3 || (!vel3.empty() && vel3.size() != pos3.size())) return false;
        const int n = (int)(pos3.size() / 3);
        std::vector<float> p4(4 * (size_t)n, 0.0f), v4(4 * (size_t)n, 0.0f);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                p4[4 * (size_t)i + k] = pos3[3 * (size_t)i + k];
                if (!vel3.empty()) v4[4 * (size_t)i + k] = vel3[3 * (size_t)i + k];
            }
        return set4(p4, v4, n);
    }

    /* -- neighbours (rx_sph_pbd.cpp:1735-1750): filled by SetParticlesToCell */
    std::vector<std::vector<rxNeigh> > &GetNeights(void) { return m_neigh; }

    /* -- the simulation space and settings (rx_ps.h:209-238) ------------ */
    Vec3 GetMax(void) const { fsph_params p = params(); return Vec3(p.box_max[0], p.box_max[1], p.box_max[2]); }
    Vec3 GetMin(void) const { fsph_params p = params(); return Vec3(p.box_min[0], p.box_min[1], p.box_min[2]); }
    Vec3 GetDim(void) const { return GetMax() - GetMin(); }
    Vec3 GetCen(void) const { return 0.5 * (GetMax() + GetMin()); }
    int GetNumParticles() const { return m_ctx ? fsph_num_particles(m_ctx) : 0; }
    int GetMaxParticles() const { return params().max_particles; }
    int GetNumBoundaryParticles() const { return m_ctx ? fsph_num_boundary(m_ctx) : 0; }
    float GetParticleRadius() const { return params().particle_radius; }
    void SetIterations(int i) {
        fsph_params p = params();
        p.max_iter = i;
        apply(p);
    }
    /* stored as in the reference, whose fluid step does not read it */
    void SetDamping(RXREAL x) { m_damping = x; }
    RXREAL GetDamping(void) const { return m_damping; }
    void SetGravity(RXREAL x) {
        m_gravity_y = x;
        if (!m_ctx) return;
        fsph_params p = params();
        p.gravity[0] = 0.0f; p.gravity[1] = x; p.gravity[2] = 0.0f;
        apply(p);
    }
    /* vorticity confinement on / off (t < 0 toggles); on uses
     * eps = kDefaultVorticityEps unless the parameters give one */
    void ToggleUseVorticity(int t = -1) {
        m_use_vorticity = t < 0 ? !m_use_vorticity : (t != 0);
        m_flags_dirty = true;
    }
    bool IsUseVorticity(void) const { return m_use_vorticity; }

    /* -- inlets and deleted particles (rx_ps.h:304; rx_ps.cpp:432-520) ---- */
    int AddLine(rxInletLine line) {
        const int k = fsph_add_inlet_line(m_ctx, line.pos1.data, line.pos2.data, line.vel.data, line.up.data,
                                          line.accum, line.span, line.spacing);
        if (k > 0) m_inlets = k;
        else m_status = -k; /* a negated status */
        return k;
    }
    /* the particles that take part in the steps (deleted ones excluded) */
    int GetNumActiveParticles() const { return m_ctx ? fsph_num_active(m_ctx) : 0; }
    /* particles strictly inside [lo, hi] at the end of a step are deleted */
    template <class V1, class V2>
    void AddDeleteRegion(const V1 &lo, const V2 &hi) {
        const Vec3 a(lo), b(hi);
        m_status = fsph_add_delete_region(m_ctx, a.data, b.data);
    }

    /* -- analytic obstacles (rx_ps.h:266-272; fsph_set_box_obstacle) ----- */
    template <class V1, class V2, class V3, class V4>
    void SetBoxObstacle(const V1 &cen, const V2 &ext, const V3 &ang, const V4 &vel, int flg) {
        const Vec3 c(cen), e(ext), a(ang), v(vel);
        m_status = fsph_set_box_obstacle(m_ctx, c.data, e.data, a.data, v.data, flg);
    }
    template <class V1, class V2>
    void SetSphereObstacle(const V1 &cen, double rad, const V2 &vel, int flg) {
        const Vec3 c(cen), v(vel);
        m_status = fsph_set_sphere_obstacle(m_ctx, c.data, rad, v.data, flg);
    }
    template <class V1>
    void MoveSphereObstacle(int b, const V1 &disp) {
        const Vec3 d(disp);
        m_status = fsph_move_sphere_obstacle(m_ctx, b, d.data);
    }
    Vec3 GetSphereObstaclePos(int b = -1) {
        Vec3 p(0.0);
        if (b < 0) b = 0;
        m_status = fsph_get_sphere_obstacle_pos(m_ctx, b, p.data);
        return p;
    }
    /* SetPolygonObstacle(vrts, nrms, tris, vel) (rx_ps.h:268): a triangle
     * mesh; the normals and the velocity are unused, as in the reference */
    template <class VV, class VN, class VT, class V1>
    void SetPolygonObstacle(const VV &vrts, const VN &nrms, const VT &tris, const V1 &vel) {
        (void)nrms;
        std::vector<double> v;
        std::vector<int> t;
        for (const auto &p : vrts) { const Vec3 q(p); v.insert(v.end(), q.data, q.data + 3); }
        for (const auto &f : tris) for (int k = 0; k < 3; ++k) t.push_back((int)f[k]);
        const Vec3 w(vel);
        m_status = fsph_set_polygon_obstacle(m_ctx, v.data(), (int)(v.size() / 3), t.data(), (int)(t.size() / 3),
                                             w.data);
    }

    /* -- density on a lattice for meshing (rx_ps.h:280-285) ------------- */
    /* hF[k n0 n1 + j n0 + i] = density at minp + (i, j, k) d (host array) */
    virtual void CalImplicitField(int n[3], Vec3 minp, Vec3 d, RXREAL *hF) {
        m_status = fsph_density_grid(m_ctx, n, minp.data, d.data, hF, FSPH_HOST);
    }
    /* the same into a device array */
    virtual void CalImplicitFieldDevice(int n[3], Vec3 minp, Vec3 d, RXREAL *dF) {
        m_status = fsph_density_grid(m_ctx, n, minp.data, d.data, dF, FSPH_DEVICE);
    }
    virtual double GetImplicit(double x, double y, double z) {
        int n[3] = {1, 1, 1};
        float v = 0.0f;
        const double p[3] = {x, y, z}, one[3] = {1.0, 1.0, 1.0};
        m_status = fsph_density_grid(m_ctx, n, p, one, &v, FSPH_HOST);
        return v;
    }

    /* -- scene set-up (rx_ps.cpp:66-261) --------------------------------- */
    void Reset(rxParticleConfig config) {
        if (!m_ctx) return;
        const int n = GetNumParticles();
        std::vector<float> p4, v4;
        get_state(p4, v4);
        if (config == RX_CONFIG_NONE) {
            m_status = fsph_set_particles(m_ctx, nullptr, nullptr, 0, FSPH_HOST);
        } else if (config == RX_CONFIG_GRID) {
            const int s = (int)std::ceil(std::pow((double)std::max(n, 1), 1.0 / 3.0));
            const double r = GetParticleRadius();
            AddBox(0, GetMin(), Vec3(s * r), Vec3(0.0), (RXREAL)(2.0 * r));
        } else { /* RX_CONFIG_RANDOM (and BOX): the particles at 2 U[0,1)^3 - 0.5 */
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) {
                    p4[4 * (size_t)i + k] = (float)(2.0 * detail::uniform01(m_seed, 3 * (uint64_t)i + k) - 0.5);
                    v4[4 * (size_t)i + k] = 0.0f;
                }
            ++m_seed;
            set4(p4, v4, n);
        }
    }
    /* AddBox(start, cen, ext, vel, spacing, attr) (rx_ps.cpp:195-261): the
     * (2 sx + 1)(2 sy + 1)(2 sz + 1) lattice around cen, sx = (int)(ext / spacing) - 1,
     * jitter 0.001 spacing; from `start` (start < 0: after the current
     * particles), wrapping to 0 past max_particles as the reference does */
    template <class V1, class V2, class V3>
    void AddBox(int start, const V1 &cen, const V2 &ext, const V3 &vel, RXREAL spacing, int attr = 0) {
        const Vec3 c(cen), e(ext), v(vel);
        const int sx = (int)(e[0] / spacing) - 1, sy = (int)(e[1] / spacing) - 1, sz = (int)(e[2] / spacing) - 1;
        const double jitter = spacing * 0.001;
        std::vector<float> pts;
        for (int z = -sz; z <= sz; ++z)
            for (int y = -sy; y <= sy; ++y)
                for (int x = -sx; x <= sx; ++x) {
                    const int dx[3] = {x, y, z};
                    for (int k = 0; k < 3; ++k)
                        pts.push_back((float)(c[k] + dx[k] * (double)spacing +
                                              (detail::uniform01(m_seed, pts.size()) * 2.0 - 1.0) * jitter));
                }
        ++m_seed;
        place(start, pts, v, attr, true);
    }
    /* AddSphere(start, pos, vel, r, spacing, attr) (rx_ps.cpp:127-193): the
     * lattice points within r spacings of pos, jitter 0.01 spacing.  As in
     * the reference, they overwrite existing particles from `start` and never
     * add beyond the current count */
    void AddSphere(int start, RXREAL *pos, RXREAL *vel, int r, RXREAL spacing, int attr = 0) {
        std::vector<float> pts;
        for (int z = -r; z <= r; ++z)
            for (int y = -r; y <= r; ++y)
                for (int x = -r; x <= r; ++x) {
                    const double d[3] = {x * (double)spacing, y * (double)spacing, z * (double)spacing};
                    if (std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) > spacing * r) continue;
                    for (int k = 0; k < 3; ++k)
                        pts.push_back((float)(pos[k] + d[k] + (detail::uniform01(m_seed, pts.size()) * 2.0 - 1.0) *
                                                                 (spacing * 0.01)));
                }
        ++m_seed;
        place(start, pts, Vec3(vel[0], vel[1], vel[2]), attr, false);
    }

    /* OutputParticles / InputParticles (rx_ps.cpp:581-644): binary
     * uint32 N, N x 3 float32 positions, N x 3 float32 velocities, no header.
     * Return 1 on success, 0 on failure, as the reference does. */
    int OutputParticles(const std::string &fn) {
        const int n = GetNumParticles();
        std::vector<float> p4, v4;
        if (n > 0 && !get_state(p4, v4)) return 0;
        FILE *f = std::fopen(fn.c_str(), "wb");
        if (!f) return 0;
        unsigned int un = (unsigned int)n;
        bool ok = std::fwrite(&un, sizeof(un), 1, f) == 1;
        for (int pass = 0; pass < 2 && ok; ++pass) {
            const std::vector<float> &a = pass ? v4 : p4;
            for (int i = 0; i < n && ok; ++i) ok = std::fwrite(&a[4 * (size_t)i], sizeof(float), 3, f) == 3;
        }
        std::fclose(f);
        return ok ? 1 : 0;
    }
    int InputParticles(const std::string &fn) {
        FILE *f = std::fopen(fn.c_str(), "rb");
        if (!f) return 0;
        unsigned int n = 0;
        if (std::fread(&n, sizeof(n), 1, f) != 1) { std::fclose(f); return 0; }
        std::vector<float> p3(3 * (size_t)n), v3(3 * (size_t)n, 0.0f);
        bool ok = std::fread(p3.data(), sizeof(float), p3.size(), f) == p3.size();
        if (ok && std::fread(v3.data(), sizeof(float), v3.size(), f) != v3.size()) std::fill(v3.begin(), v3.end(), 0.0f);
        std::fclose(f);
        return ok && Set(p3, v3) ? 1 : 0;
    }

    /* Checkpoint: the reference's particle file at fn (OutputParticles), the
     * exact device state at fn + ".state" (fsph_save_state) and a JSON
     * sidecar at fn + ".json" with the parameters and the placement RNG
     * seed (the AddBox / AddSphere / AddLine jitter counter).  LoadCheckpoint
     * resumes bit-identically to continuing without the checkpoint; without
     * the ".state" file it falls back to the particle file (the seed is
     * still restored).  Return 1 on success, 0 on failure. */
    int SaveCheckpoint(const std::string &fn) {
        if (!m_ctx || !OutputParticles(fn)) return 0;
        m_status = fsph_save_state(m_ctx, (fn + ".state").c_str());
        if (m_status != FSPH_OK) return 0;
        const fsph_params p = params();
        std::string state; /* the state file's name as a JSON string body */
        for (char ch : fn + ".state") {
            if (ch == '"' || ch == '\\') state.push_back('\\');
            state.push_back(ch);
        }
        FILE *f = std::fopen((fn + ".json").c_str(), "w");
        if (!f) return 0;
        std::fprintf(f,
                     "{\"format\": \"fsph checkpoint 1\", \"solver\": %d, \"particles\": %d, "
                     "\"active\": %d, \"max_particles\": %d, \"seed\": %llu, \"inlets\": %d, "
                     "\"h\": %.9g, \"mass\": %.9g, \"rest_dens\": %.9g, \"dt_note\": \"dt is an Update argument\", "
                     "\"box_min\": [%.17g, %.17g, %.17g], \"box_max\": [%.17g, %.17g, %.17g], "
                     "\"state\": \"%s\"}\n",
                     p.solver, GetNumParticles(), GetNumActiveParticles(), p.max_particles,
                     (unsigned long long)m_seed, m_inlets, (double)p.h, (double)p.mass, (double)p.rest_dens,
                     p.box_min[0], p.box_min[1], p.box_min[2], p.box_max[0], p.box_max[1], p.box_max[2], state.c_str());
        const bool ok = std::fclose(f) == 0;
        return ok ? 1 : 0;
    }
    int LoadCheckpoint(const std::string &fn) {
        if (!m_ctx) return 0;
        FILE *f = std::fopen((fn + ".json").c_str(), "r");
        if (f) { /* the seed and the inlet count from the sidecar */
            char buf[4096];
            const size_t k = std::fread(buf, 1, sizeof(buf) - 1, f);
            std::fclose(f);
            buf[k] = 0;
            const char *q = std::strstr(buf, "\"seed\": ");
            if (q) m_seed = std::strtoull(q + 8, nullptr, 10);
            q = std::strstr(buf, "\"inlets\": ");
            if (q) m_inlets = (int)std::strtol(q + 10, nullptr, 10);
        }
        m_status = fsph_load_state(m_ctx, (fn + ".state").c_str());
        if (m_status == FSPH_OK) {
            m_inlets = fsph_num_inlets(m_ctx);
            const fsph_params p = params();
            m_use_vorticity = p.vort_eps != 0.0f;
            m_artificial_pressure = p.use_ap != 0;
            m_gravity_y = p.gravity[1];
            return 1;
        }
        return InputParticles(fn);
    }

    /* g_iIterations / g_fEta of the last step (rx_sph_pbd.cpp:461-462) */
    int GetIterations() const { return m_stats.iterations; }
    float GetDensityError() const { return m_stats.density_error; }
    const fsph_step_stats &GetStepStats() const { return m_stats; }
    /* one JSON line per step appended to `path` (nullptr stops) */
    bool SetStepLog(const char *path) {
        m_status = m_ctx ? fsph_set_step_log(m_ctx, path) : FSPH_NOT_INITIALIZED;
        return m_status == FSPH_OK;
    }
    fsph_ctx *Context() { return m_ctx; }

    static constexpr float kDefaultVorticityEps = 1e-4f;

protected:
    /* -- step ---------------------------------------------------------- */
    bool update_impl(RXREAL dt, int step) {
        /* the inlet lines due at this step first (rx_sph_pbd_gpu.cpp:795-815) */
        if (m_ctx && m_inlets) {
            m_status = fsph_emit_inlets(m_ctx, step, nullptr);
            if (m_status != FSPH_OK) return false;
        }
        if (!m_ctx || fsph_num_particles(m_ctx) == 0) return false;
        sync_flags();
        m_status = fsph_step(m_ctx, dt, nullptr, &m_stats);
        return m_status == FSPH_OK;
    }
    bool fields_impl(RXREAL dt) {
        if (!m_ctx || fsph_num_particles(m_ctx) == 0) return false;
        sync_flags();
        m_status = fsph_step_fields(m_ctx, dt, nullptr);
        return m_status == FSPH_OK;
    }

    /* SetArrayVBO(type, data, start, count) (rx_ps.h:260-262), DIM = 4 stride */
    void set_array_impl(rxParticleArray type, const void *data, int start, int count) {
        m_status = fsph_set_array(m_ctx, (int)type, data, start, count, FSPH_HOST);
    }

    /* GetArrayVBO(type, d2h, num) (rx_ps.h:259): non-owning host pointer, or
     * nullptr for an array the fluid step does not hold */
    RXREAL *get_array_impl(rxParticleArray type, bool d2h, int num) {
        (void)num;
        const int n = GetNumParticles();
        const bool vec = type == RX_POSITION || type == RX_VELOCITY || type == RX_FORCE ||
                         type == RX_PREDICT_POS || type == RX_CORRECTION || type == RX_VORTICITY;
        const bool held = vec || type == RX_DENSITY || type == RX_PRESSURE || type == RX_ATTRIBUTE ||
                          type == RX_SCALING_FACTOR;
        if (!held) return nullptr;
        std::vector<float> &buf = m_host[(int)type % kSlots];
        buf.resize((size_t)std::max(n, 1) * (vec ? 4 : 1));
        if (d2h && n > 0) m_status = fsph_get_array(m_ctx, (int)type, buf.data(), FSPH_HOST, nullptr);
        return buf.data();
    }
    static const int kSlots = 64;
    int m_solver;
    fsph_ctx *m_ctx = nullptr;
    int m_status = FSPH_NOT_INITIALIZED;
    fsph_step_stats m_stats{};
    std::vector<float> m_host[kSlots];
    std::vector<std::vector<rxNeigh> > m_neigh;
    RXREAL m_damping = 0.0f;
    RXREAL m_gravity_y = -9.82f;
    bool m_use_vorticity = false;
    bool m_artificial_pressure = true;
    bool m_flags_dirty = false;
    int m_inlets = 0;
    uint64_t m_seed = 1;

    void create(const fsph_params &p) {
        if (m_ctx) { fsph_destroy(m_ctx); m_ctx = nullptr; }
        fsph_params q = p;
        q.solver = m_solver;
        m_status = fsph_create(&q, &m_ctx);
        if (m_status != FSPH_OK) { m_ctx = nullptr; return; }
        m_use_vorticity = q.vort_eps != 0.0f;
        m_artificial_pressure = q.use_ap != 0;
        m_gravity_y = q.gravity[1];
    }
    fsph_params params() const {
        fsph_params p;
        if (!m_ctx || fsph_get_params(m_ctx, &p) != FSPH_OK) fsph_params_default(&p);
        return p;
    }
    void apply(const fsph_params &p) {
        if (m_ctx) m_status = fsph_set_params(m_ctx, &p);
    }
    /* flags a caller may flip between steps (vorticity, GetArtificialPressure) */
    void sync_flags() {
        fsph_params p = params();
        const bool vort = p.vort_eps != 0.0f;
        const bool ap = p.use_ap != 0;
        if (vort == m_use_vorticity && ap == m_artificial_pressure && !m_flags_dirty) return;
        p.vort_eps = m_use_vorticity ? (vort ? p.vort_eps : kDefaultVorticityEps) : 0.0f;
        p.use_ap = m_artificial_pressure ? 1 : 0;
        m_flags_dirty = false;
        if (vort != m_use_vorticity || ap != m_artificial_pressure) apply(p);
    }
    bool set4(const std::vector<float> &p4, const std::vector<float> &v4, int n) {
        m_status = fsph_set_particles(m_ctx, n ? p4.data() : nullptr, n ? v4.data() : nullptr, n, FSPH_HOST);
        return m_status == FSPH_OK;
    }
    bool get_state(std::vector<float> &p4, std::vector<float> &v4) {
        const int n = GetNumParticles();
        p4.assign(4 * (size_t)n, 0.0f);
        v4.assign(4 * (size_t)n, 0.0f);
        if (n == 0) return true;
        m_status = fsph_get_array(m_ctx, FSPH_POSITION, p4.data(), FSPH_HOST, nullptr);
        if (m_status == FSPH_OK) m_status = fsph_get_array(m_ctx, FSPH_VELOCITY, v4.data(), FSPH_HOST, nullptr);
        return m_status == FSPH_OK;
    }
    /* write particles xyz[] (with velocity vel, attribute attr) from `start`;
     * grow: the count may grow (AddBox), else only existing ones change */
    void place(int start, const std::vector<float> &xyz, const Vec3 &vel, int attr, bool grow) {
        if (!m_ctx) return;
        const int n0 = GetNumParticles(), cap = GetMaxParticles();
        std::vector<float> p4, v4;
        if (!get_state(p4, v4)) return;
        std::vector<int> at((size_t)n0, 0);
        if (n0 > 0) m_status = fsph_get_array(m_ctx, FSPH_ATTRIBUTE, at.data(), FSPH_HOST, nullptr);
        int index = start < 0 ? n0 : start;
        int n = n0;
        bool over = false;
        const int count = (int)(xyz.size() / 3);
        for (int q = 0; q < count; ++q) {
            if (index >= cap) { index = 0; over = true; }
            if (!grow && index >= n0) break;
            if (index >= n) {
                n = index + 1;
                p4.resize(4 * (size_t)n, 0.0f);
                v4.resize(4 * (size_t)n, 0.0f);
                at.resize((size_t)n, 0);
            }
            for (int k = 0; k < 3; ++k) {
                p4[4 * (size_t)index + k] = xyz[3 * (size_t)q + k];
                v4[4 * (size_t)index + k] = (float)vel[k];
            }
            p4[4 * (size_t)index + 3] = v4[4 * (size_t)index + 3] = 0.0f;
            at[(size_t)index] = attr;
            ++index;
        }
        if (over) n = cap;
        p4.resize(4 * (size_t)n, 0.0f);
        v4.resize(4 * (size_t)n, 0.0f);
        at.resize((size_t)n, 0);
        if (!set4(p4, v4, n) || n == 0) return;
        m_status = fsph_set_array(m_ctx, FSPH_ATTRIBUTE, at.data(), 0, n, FSPH_HOST);
    }
    void neighbours(const RXREAL *prts, int n, RXREAL h) {
        std::vector<float> p4;
        if (prts) { /* DIM = 4 stride, as the reference's arrays */
            p4.assign(prts, prts + 4 * (size_t)n);
        }
        const int rows = prts ? n : GetNumParticles();
        std::vector<int> off((size_t)rows + 1, 0);
        long long total = 0;
        m_status = fsph_neighbors_ex(m_ctx, prts ? p4.data() : nullptr, n, h, FSPH_HOST, off.data(), nullptr,
                                     nullptr, 0, &total);
        if (m_status != FSPH_OK) return;
        std::vector<int> idx((size_t)std::max(total, 1LL));
        std::vector<float> d2((size_t)std::max(total, 1LL));
        m_status = fsph_neighbors_ex(m_ctx, prts ? p4.data() : nullptr, n, h, FSPH_HOST, off.data(), idx.data(),
                                     d2.data(), total, &total);
        if (m_status != FSPH_OK) return;
        m_neigh.assign((size_t)rows, {});
        for (int i = 0; i < rows; ++i)
            for (int k = off[i]; k < off[i + 1]; ++k)
                m_neigh[i].push_back(rxNeigh{idx[k], std::sqrt(d2[k]), d2[k]});
    }
};

/* The pure virtuals of rx_ps.h:253-275 over the C ABI, common to both solvers. */
class rxFsphSolver : public rxParticleSystemBase {
public:
    using rxParticleSystemBase::rxParticleSystemBase;
    bool Update(RXREAL dt, int step = 0) override { return update_impl(dt, step); }
    bool UpdateWithoutPosAndVel(RXREAL dt, int step = 0) override {
        (void)step;
        return fields_impl(dt);
    }
    RXREAL *GetArrayVBO(rxParticleArray type, bool d2h = true, int num = -1) override {
        return get_array_impl(type, d2h, num);
    }
    void SetArrayVBO(rxParticleArray type, const RXREAL *data, int start, int count) override {
        set_array_impl(type, data, start, count);
    }
    void SetArrayVBO(rxParticleArray type, const int *data, int start, int count) override {
        set_array_impl(type, data, start, count);
    }
    RXREAL *GetParticle(void) override { return get_array_impl(RX_POSITION, true, -1); }
    RXREAL *GetParticleDevice(void) override { return (RXREAL *)fsph_device_ptr(m_ctx, FSPH_POSITION); }
    void SetParticlesToCell(void) override { neighbours(nullptr, 0, -1.0f); }
    void SetParticlesToCell(RXREAL *prts, int n, RXREAL h) override { neighbours(prts, n, h); }
};

/* Weakly compressible SPH (rxSPH / rxSPH_GPU). */
class rxSPH : public rxFsphSolver {
public:
    explicit rxSPH(bool use_opengl = false) : rxFsphSolver(FSPH_SOLVER_WCSPH, use_opengl) {}
    explicit rxSPH(const fsph_params &p) : rxFsphSolver(p, FSPH_SOLVER_WCSPH) {}
};

/* Position Based Fluids (rxPBDSPH / rxPBDSPH_GPU). */
class rxPBDSPH : public rxFsphSolver {
public:
    explicit rxPBDSPH(bool use_opengl = false) : rxFsphSolver(FSPH_SOLVER_PBF, use_opengl) {}
    explicit rxPBDSPH(const fsph_params &p) : rxFsphSolver(p, FSPH_SOLVER_PBF) {}
    /* the tensile-instability term on / off (rx_sph.h:1199), read at the next Update */
    bool &GetArtificialPressure(void) { return m_artificial_pressure; }
    /* Static boundary particles, 4 floats each (the boundary set-up of
     * rxPBDSPH::Initialize, rx_sph_pbd.cpp:280-297); an empty vector removes them. */
    bool SetBoundary(const std::vector<float> &bpos4) {
        const int nb = (int)(bpos4.size() / 4);
        m_status = fsph_set_boundary(m_ctx, nb ? bpos4.data() : nullptr, nb, FSPH_HOST);
        return m_status == FSPH_OK;
    }
    /* positions (4 floats each), psi_b or lambda_b, in the given order */
    std::vector<float> GetBoundary(int which) {
        std::vector<float> out((size_t)GetNumBoundaryParticles() * (which == FSPH_BOUNDARY_POSITION ? 4 : 1));
        if (!out.empty()) m_status = fsph_get_boundary(m_ctx, which, out.data());
        return out;
    }
    /* The learned warm start (no counterpart in the reference): a network
     * blob of FSPH_MLP_BLOB_SIZE floats (the layout of fsph.h), used by the
     * steps while the parameters have warm_start = 1. */
    bool SetWarmStartModel(const std::vector<float> &blob) {
        if (blob.size() != (size_t)FSPH_MLP_BLOB_SIZE) {
            m_status = FSPH_INVALID_ARG;
            return false;
        }
        m_status = fsph_set_warm_start_model(m_ctx, blob.data());
        return m_status == FSPH_OK;
    }
    /* Initialize(env) derivation (rx_sph_pbd.cpp:102-201) without a context */
    static fsph_params ParamsFromEnv(const fsph_env &env) {
        fsph_params p;
        fsph_params_from_env(&env, &p);
        return p;
    }
};

}  // namespace fsph_gb300
