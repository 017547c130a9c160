/*
 * A caller written the way the reference's application drives its particle
 * system (rxFlGLWindow::InitSPH / StepPS, rx_fltk_glcanvas.cpp:2386-2496, and
 * rxSPHConfig::SetLiquidBox -> AddBox, rx_sph_config.h:257-269), compiled
 * against fsph_particle_system.hpp without changes beyond the include and
 * the namespace: a base-class pointer, the two-phase Initialize(env), the
 * scene set-up, the step loop with SetIterations / SetDamping / SetGravity /
 * Update, then the neighbour lists, UpdateWithoutPosAndVel and the particle
 * file.  Prints one summary line; used by tests/test_gpu_cpp_mirror.py.
 *
 *   ref_style_caller out.dat steps
 */
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "fsph_particle_system.hpp"

using namespace fsph_gb300;
#define RXSPH rxPBDSPH

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s out.dat steps\n", argv[0]);
        return 2;
    }
    const auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](const char *what) { /* phase times on stderr */
        std::fprintf(stderr, "%s %.3f s\n", what,
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    };
    rxParticleSystemBase *m_pPS = new RXSPH(true);

    // InitSPH: the scene's environment, then Initialize
    rxSPHEnviroment sph_env;
    sph_env.max_particles = 20000;
    sph_env.boundary_cen = Vec3(0.0, 0.0, 0.0);
    sph_env.boundary_ext = Vec3(0.8, 0.4, 0.4);
    sph_env.dens = (RXREAL)998.29;
    sph_env.mass = (RXREAL)0.02;  // h = 0.0457 (kernel_particles 20); at h = 0.01 the reference's dt^2-scaled
                                  // tensile correction outweighs lambda and the block explodes
    sph_env.kernel_particles = (RXREAL)20.0;
    sph_env.dt = (RXREAL)0.002;
    sph_env.epsilon = (RXREAL)100.0;
    sph_env.eta = (RXREAL)0.01;
    sph_env.min_iter = 2;
    sph_env.max_iter = 10;
    ((RXSPH *)m_pPS)->Initialize(sph_env);
    if (!((RXSPH *)m_pPS)->IsInitialized()) {
        std::fprintf(stderr, "Initialize: %s\n", ((RXSPH *)m_pPS)->LastError().c_str());
        return 1;
    }
    const double m_fDt = sph_env.dt;
    lap("initialized");
    m_pPS->ToggleUseVorticity(0);
    m_pPS->Reset(rxParticleSystemBase::RX_CONFIG_NONE);

    // SetLiquidBox: a block of fluid in the lower corner of the box
    RXREAL pr = m_pPS->GetParticleRadius();
    Vec3 cen = m_pPS->GetMin() + Vec3(0.25, 0.25, 0.25);
    m_pPS->AddBox(-1, cen, Vec3(0.2, 0.2, 0.2), Vec3(0.0), pr * 2.0f);
    const int n0 = m_pPS->GetNumParticles();
    if (n0 <= 0) { std::fprintf(stderr, "AddBox placed no particles\n"); return 1; }
    // a polygon obstacle as the scene loader hands one over (vertices, normals, index triples)
    {
        std::vector<Vec3> vrts = {m_pPS->GetMax() - Vec3(0.1, 0.1, 0.1), m_pPS->GetMax() - Vec3(0.02, 0.1, 0.1),
                                  m_pPS->GetMax() - Vec3(0.1, 0.02, 0.1)};
        std::vector<Vec3> nrms(3, Vec3(0.0, 0.0, 1.0));
        std::vector<std::vector<int> > tris = {{0, 1, 2}};
        m_pPS->SetPolygonObstacle(vrts, nrms, tris, Vec3(0.0));
        if (m_pPS->LastStatus() != FSPH_OK) { std::fprintf(stderr, "SetPolygonObstacle failed\n"); return 1; }
    }
    lap("scene placed");

    // StepPS
    const int steps = std::atoi(argv[2]);
    for (int m_iCurrentStep = 0; m_iCurrentStep < steps; ++m_iCurrentStep) {
        float damping = 1.0f;
        int iterations = 10;
        m_pPS->SetIterations(iterations);
        m_pPS->SetDamping(damping);
        m_pPS->SetGravity((RXREAL)(-9.8));
        if (!m_pPS->Update((RXREAL)m_fDt, m_iCurrentStep)) {
            std::fprintf(stderr, "Update failed at step %d\n", m_iCurrentStep);
            return 1;
        }
    }

    lap("stepped");
    // neighbour lists of the current positions
    m_pPS->SetParticlesToCell();
    const std::vector<std::vector<rxNeigh> > &nb = ((RXSPH *)m_pPS)->GetNeights();
    size_t total = 0;
    double worst = 0.0;
    for (const std::vector<rxNeigh> &row : nb)
        for (const rxNeigh &q : row) {
            ++total;
            worst = std::fmax(worst, std::fabs((double)q.Dist * q.Dist - q.Dist2) / std::fmax(q.Dist2, 1e-30f));
        }

    // the fields of a step without moving the particles
    RXREAL *x = m_pPS->GetArrayVBO(rxParticleSystemBase::RX_POSITION);
    const double x0 = x[0];
    if (!m_pPS->UpdateWithoutPosAndVel((RXREAL)m_fDt, steps)) { std::fprintf(stderr, "fields failed\n"); return 1; }
    x = m_pPS->GetArrayVBO(rxParticleSystemBase::RX_POSITION);
    const int unmoved = x[0] == x0 ? 1 : 0; /* read now: the resume check below steps the system on */
    RXREAL *rho = m_pPS->GetArrayVBO(rxParticleSystemBase::RX_DENSITY);
    double rmin = 1e30, rmax = 0.0;
    for (int i = 0; i < m_pPS->GetNumParticles(); ++i) {
        rmin = std::fmin(rmin, (double)rho[i]);
        rmax = std::fmax(rmax, (double)rho[i]);
    }

    lap("neighbours and fields");
    // the particle file
    if (!m_pPS->OutputParticles(argv[1])) { std::fprintf(stderr, "OutputParticles failed\n"); return 1; }
    // a checkpoint: a second system resumed from it steps as this one does
    const std::string ckpt = std::string(argv[1]) + ".ckpt";
    if (!m_pPS->SaveCheckpoint(ckpt)) { std::fprintf(stderr, "SaveCheckpoint failed\n"); return 1; }
    rxParticleSystemBase *resumed = new RXSPH(true);
    ((RXSPH *)resumed)->Initialize(sph_env);
    if (!resumed->LoadCheckpoint(ckpt)) { std::fprintf(stderr, "LoadCheckpoint failed\n"); return 1; }
    for (int k = 0; k < 5; ++k) {
        m_pPS->Update((RXREAL)m_fDt, steps + 1 + k);
        resumed->Update((RXREAL)m_fDt, steps + 1 + k);
    }
    const int n = m_pPS->GetNumParticles();
    std::vector<RXREAL> xa(m_pPS->GetArrayVBO(rxParticleSystemBase::RX_POSITION),
                           m_pPS->GetArrayVBO(rxParticleSystemBase::RX_POSITION, false) + 4 * (size_t)n);
    const RXREAL *xr = resumed->GetArrayVBO(rxParticleSystemBase::RX_POSITION);
    int same = resumed->GetNumParticles() == n ? 1 : 0;
    for (size_t k = 0; same && k < xa.size(); ++k) same = xa[k] == xr[k] ? 1 : 0;
    delete resumed;
    std::printf("particles %d max %d neighbours %zu dist_check %.3e unmoved %d density %.3f %.3f dim %.3f %.3f %.3f"
                " resume %d\n",
                m_pPS->GetNumParticles(), m_pPS->GetMaxParticles(), total, worst, unmoved, rmin, rmax,
                m_pPS->GetDim()[0], m_pPS->GetDim()[1], m_pPS->GetDim()[2], same);
    delete m_pPS;
    return 0;
}
