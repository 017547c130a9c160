/*
 * fsph_particle_system.hpp -- C++ drop-in for the reference's particle-system
 * classes, over the C ABI of fsph.h (header only; link libfsph.so).
 *
 * Same class and method names as rxParticleSystemBase (rx_ps.h:55-333),
 * rxSPH (rx_sph.h:202-426) and rxPBDSPH (rx_sph.h:1027-1274), with the same
 * argument meaning and error behaviour:
 *   - Update returns false when there is nothing to step (N = 0), as
 *     rxPBDSPH_GPU::Update does (rx_sph_pbd_gpu.cpp:818);
 *   - GetArrayVBO returns a NON-OWNING pointer to an internal host buffer,
 *     refreshed from the device when d2h is true (rx_sph_pbd_gpu.cpp:2497-2613),
 *     vectors with the DIM = 4 stride;
 *   - GetParticleDevice returns a borrowed device pointer (device order; the
 *     reference's CPU class returned a fresh copy the caller freed,
 *     rx_sph_pbd.cpp:499-509);
 *   - GetNeights returns the neighbour lists (particle indices) of the
 *     current positions (rx_sph.h:1196).
 * The status of the last failing call is LastStatus() / LastError().
 * GL-only members (SetColorVBO, Draw*, VBO ids) do not exist here.
 */
#pragma once

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fsph.h"

namespace fsph_gb300 {

class rxParticleSystemBase {
public:
    enum rxParticleArray {
        RX_POSITION = FSPH_POSITION,
        RX_VELOCITY = FSPH_VELOCITY,
        RX_FORCE = FSPH_FORCE,
        RX_DENSITY = FSPH_DENSITY,
        RX_PRESSURE = FSPH_PRESSURE,
        RX_ATTRIBUTE = FSPH_ATTRIBUTE,
        RX_PREDICT_POS = FSPH_PREDICT_POS,
        RX_SCALING_FACTOR = FSPH_SCALING_FACTOR,
        RX_CORRECTION = FSPH_CORRECTION,
        RX_VORTICITY = FSPH_VORTICITY
    };

    explicit rxParticleSystemBase(const fsph_params &p, int solver) {
        fsph_params q = p;
        q.solver = solver;
        m_status = fsph_create(&q, &m_ctx);
    }
    virtual ~rxParticleSystemBase() {
        if (m_ctx) fsph_destroy(m_ctx);
    }
    rxParticleSystemBase(const rxParticleSystemBase &) = delete;
    rxParticleSystemBase &operator=(const rxParticleSystemBase &) = delete;

    bool IsInitialized() const { return m_ctx != nullptr; }
    int LastStatus() const { return m_status; }
    std::string LastError() const { return m_ctx ? fsph_last_error(m_ctx) : fsph_status_string(m_status); }

    /* Update(dt, step) (rx_ps.h:254) */
    virtual bool Update(float dt, int step = 0) {
        (void)step;
        if (!m_ctx || fsph_num_particles(m_ctx) == 0) return false;
        m_status = fsph_step(m_ctx, dt, nullptr, &m_stats);
        return m_status == FSPH_OK;
    }

    /* Set(ppos, pvel) (rx_ps.cpp:30-59): xyz triples, sizes must agree */
    bool Set(const std::vector<float> &pos3, const std::vector<float> &vel3) {
        if (pos3.empty() || pos3.size() % 3 || (!vel3.empty() && vel3.size() != pos3.size())) return false;
        const int n = (int)(pos3.size() / 3);
        std::vector<float> p4(4 * (size_t)n, 0.0f), v4(4 * (size_t)n, 0.0f);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                p4[4 * (size_t)i + k] = pos3[3 * (size_t)i + k];
                if (!vel3.empty()) v4[4 * (size_t)i + k] = vel3[3 * (size_t)i + k];
            }
        m_status = fsph_set_particles(m_ctx, p4.data(), v4.data(), n, FSPH_HOST);
        return m_status == FSPH_OK;
    }

    /* SetArrayVBO(type, data, start, count) (rx_ps.h:260-262), DIM = 4 stride */
    void SetArrayVBO(rxParticleArray type, const float *data, int start, int count) {
        m_status = fsph_set_array(m_ctx, (int)type, data, start, count, FSPH_HOST);
    }
    void SetArrayVBO(rxParticleArray type, const int *data, int start, int count) {
        m_status = fsph_set_array(m_ctx, (int)type, data, start, count, FSPH_HOST);
    }

    /* GetArrayVBO(type, d2h, num) (rx_ps.h:259): non-owning host pointer */
    float *GetArrayVBO(rxParticleArray type, bool d2h = true, int num = -1) {
        (void)num;
        const int n = GetNumParticles();
        const bool vec = type == RX_POSITION || type == RX_VELOCITY || type == RX_FORCE ||
                         type == RX_PREDICT_POS || type == RX_CORRECTION || type == RX_VORTICITY;
        std::vector<float> &buf = m_host[(int)type % kSlots];
        buf.resize((size_t)n * (vec ? 4 : 1));
        if (d2h && n > 0) m_status = fsph_get_array(m_ctx, (int)type, buf.data(), FSPH_HOST, nullptr);
        return buf.data();
    }

    float *GetParticle() { return GetArrayVBO(RX_POSITION); }
    float *GetParticleDevice() { return (float *)fsph_device_ptr(m_ctx, FSPH_POSITION); }

    int GetNumParticles() const { return m_ctx ? fsph_num_particles(m_ctx) : 0; }
    int GetMaxParticles() const { fsph_params p; fsph_get_params(m_ctx, &p); return p.max_particles; }
    float GetParticleRadius() const { fsph_params p; fsph_get_params(m_ctx, &p); return p.particle_radius; }

    /* SetGravity / SetIterations (rx_ps.h:220-227) */
    void SetGravity(float x) {
        fsph_params p;
        fsph_get_params(m_ctx, &p);
        p.gravity[0] = 0.0f; p.gravity[1] = x; p.gravity[2] = 0.0f;
        m_status = fsph_set_params(m_ctx, &p);
    }
    void SetIterations(int i) {
        fsph_params p;
        fsph_get_params(m_ctx, &p);
        p.max_iter = i;
        m_status = fsph_set_params(m_ctx, &p);
    }

    /* SetParticlesToCell + GetNeights (rx_sph.h:1196) */
    void SetParticlesToCell() {
        const int n = GetNumParticles();
        std::vector<int> off((size_t)n + 1);
        long long total = 0;
        m_status = fsph_neighbors(m_ctx, off.data(), nullptr, 0, &total);
        if (m_status != FSPH_OK) return;
        std::vector<int> idx((size_t)(total > 0 ? total : 1));
        m_status = fsph_neighbors(m_ctx, off.data(), idx.data(), total, &total);
        m_neigh.assign((size_t)n, {});
        for (int i = 0; i < n; ++i) m_neigh[i].assign(idx.begin() + off[i], idx.begin() + off[i + 1]);
    }
    std::vector<std::vector<int> > &GetNeights() { return m_neigh; }

    /* OutputParticles / InputParticles (rx_ps.cpp:581-644): binary
     * uint32 N, N x 3 float32 positions, N x 3 float32 velocities, no header.
     * Return 1 on success, 0 on failure, as the reference does. */
    int OutputParticles(const std::string &fn) {
        const int n = GetNumParticles();
        std::vector<float> p4(4 * (size_t)n), v4(4 * (size_t)n);
        if (n > 0 && (fsph_get_array(m_ctx, FSPH_POSITION, p4.data(), FSPH_HOST, nullptr) != FSPH_OK ||
                      fsph_get_array(m_ctx, FSPH_VELOCITY, v4.data(), FSPH_HOST, nullptr) != FSPH_OK))
            return 0;
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

    /* g_iIterations / g_fEta of the last step (rx_sph_pbd.cpp:461-462) */
    int GetIterations() const { return m_stats.iterations; }
    float GetDensityError() const { return m_stats.density_error; }
    const fsph_step_stats &GetStepStats() const { return m_stats; }
    fsph_ctx *Context() { return m_ctx; }

protected:
    static const int kSlots = 32;
    fsph_ctx *m_ctx = nullptr;
    int m_status = FSPH_NOT_INITIALIZED;
    fsph_step_stats m_stats{};
    std::vector<float> m_host[kSlots];
    std::vector<std::vector<int> > m_neigh;
};

/* Weakly compressible SPH (rxSPH / rxSPH_GPU). */
class rxSPH : public rxParticleSystemBase {
public:
    explicit rxSPH(const fsph_params &p) : rxParticleSystemBase(p, FSPH_SOLVER_WCSPH) {}
};

/* Position Based Fluids (rxPBDSPH / rxPBDSPH_GPU). */
class rxPBDSPH : public rxParticleSystemBase {
public:
    explicit rxPBDSPH(const fsph_params &p) : rxParticleSystemBase(p, FSPH_SOLVER_PBF) {}
    /* Static boundary particles, 4 floats each (the boundary set-up of
     * rxPBDSPH::Initialize, rx_sph_pbd.cpp:280-297); an empty vector removes them. */
    bool SetBoundary(const std::vector<float> &bpos4) {
        const int nb = (int)(bpos4.size() / 4);
        m_status = fsph_set_boundary(m_ctx, nb ? bpos4.data() : nullptr, nb, FSPH_HOST);
        return m_status == FSPH_OK;
    }
    int GetNumBoundaryParticles() const { return m_ctx ? fsph_num_boundary(m_ctx) : 0; }
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
    /* Initialize(env) derivation (rx_sph_pbd.cpp:102-201) */
    static fsph_params ParamsFromEnv(const fsph_env &env) {
        fsph_params p;
        fsph_params_from_env(&env, &p);
        return p;
    }
};

}  // namespace fsph_gb300
