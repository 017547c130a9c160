/*
 * Test-infrastructure C ABI over the reference's own CPU fluid functions
 * (compiled into oracle/_ref/libfsph_ref.so by extract.py).  Only the oracle
 * tests and the CPU-baseline leg of the benchmark load it.
 *
 * Allocate() mirrors rxPBDSPH::Allocate / rxSPH::Allocate
 * (rx_sph_pbd.cpp:208-331, rx_sph_cpu.cpp): zeroed host arrays of
 * max_particles * DIM floats and a grid Setup over the expanded domain, minus
 * the VBOs and the anisotropic-kernel buffers.
 */
#include <cstdint>

rxPBDSPH::~rxPBDSPH() {
    delete[] m_hPos; delete[] m_hVel; delete[] m_hNrm; delete[] m_hFrc;
    delete[] m_hDens; delete[] m_hPres; delete[] m_hS; delete[] m_hDp;
    delete[] m_hPredictPos; delete[] m_hPredictVel;
    delete m_pBoundary;
    delete m_pNNGrid;
}

void rxPBDSPH::Allocate(int max_particles) {
    m_uMaxParticles = max_particles;
    size_t size = (size_t)m_uMaxParticles * DIM, size1 = m_uMaxParticles;
    m_hPos = new RXREAL[size](); m_hVel = new RXREAL[size](); m_hNrm = new RXREAL[size]();
    m_hFrc = new RXREAL[size](); m_hDens = new RXREAL[size1](); m_hPres = new RXREAL[size1]();
    m_hS = new RXREAL[size1](); m_hDp = new RXREAL[size]();
    m_hPredictPos = new RXREAL[size](); m_hPredictVel = new RXREAL[size]();
    m_vNeighs.resize(m_uMaxParticles);
    m_pNNGrid->Setup(m_v3EnvMin, m_v3EnvMax, m_fEffectiveRadius, m_uMaxParticles);
    m_bInitialized = true;
}

rxSPH::~rxSPH() {
    delete[] m_hPos; delete[] m_hVel; delete[] m_hNrm; delete[] m_hFrc;
    delete[] m_hDens; delete[] m_hPres;
    delete m_pBoundary;
    delete m_pNNGrid;
}

void rxSPH::Allocate(int max_particles) {
    m_uMaxParticles = max_particles;
    size_t size = (size_t)m_uMaxParticles * DIM, size1 = m_uMaxParticles;
    m_hPos = new RXREAL[size](); m_hVel = new RXREAL[size](); m_hNrm = new RXREAL[size]();
    m_hFrc = new RXREAL[size](); m_hDens = new RXREAL[size1](); m_hPres = new RXREAL[size1]();
    m_vNeighs.resize(m_uMaxParticles);
    m_pNNGrid->Setup(m_v3EnvMin, m_v3EnvMax, m_fEffectiveRadius, m_uMaxParticles);
    m_bInitialized = true;
}

/* Scene / solver description handed over by the tests. */
typedef struct {
    int max_particles;
    double boundary_cen[3];
    double boundary_ext[3];
    float dens, mass, kernel_particles, viscosity, gas_k;
    float epsilon, eta;
    int min_iter, max_iter;
    int use_ap;
    float ap_k, ap_n, ap_q;
    /* explicit overrides of derived values; <= 0 keeps the derived value */
    float h, particle_radius, rest_dens;
    float gravity_y;
} fsph_ref_env;

static rxSPHEnviroment make_env(const fsph_ref_env *e) {
    rxSPHEnviroment env;
    env.max_particles = e->max_particles;
    env.boundary_cen = Vec3(e->boundary_cen[0], e->boundary_cen[1], e->boundary_cen[2]);
    env.boundary_ext = Vec3(e->boundary_ext[0], e->boundary_ext[1], e->boundary_ext[2]);
    env.dens = e->dens; env.mass = e->mass; env.kernel_particles = e->kernel_particles;
    env.viscosity = e->viscosity; env.gas_k = e->gas_k;
    env.epsilon = e->epsilon; env.eta = e->eta; env.min_iter = e->min_iter; env.max_iter = e->max_iter;
    env.use_ap = e->use_ap; env.ap_k = e->ap_k; env.ap_n = e->ap_n; env.ap_q = e->ap_q;
    return env;
}

template <class S>
static void apply_overrides(S *s, const fsph_ref_env *e) {
    bool regrid = false;
    if (e->h > 0) {
        s->m_fEffectiveRadius = e->h;
        s->m_fKernelRadius = e->h;
        RXREAL h = s->m_fEffectiveRadius;
        s->m_fAw = KernelCoefPoly6(h, 3, 1);
        s->m_fAg = KernelCoefSpiky(h, 3, 2);
        s->m_fAl = KernelCoefVisc(h, 3, 3);
        regrid = true;
    }
    if (e->particle_radius > 0) s->m_fParticleRadius = e->particle_radius;
    if (e->rest_dens > 0) s->m_fRestDens = e->rest_dens;
    else if (e->h > 0 || e->particle_radius > 0) s->m_fRestDens = s->calRestDensity(s->m_fEffectiveRadius);
    s->SetGravity(e->gravity_y);
    if (regrid) {
        delete s->m_pNNGrid;
        s->m_pNNGrid = new rxNNGrid(DIM);
        s->m_pNNGrid->Setup(s->m_v3EnvMin, s->m_v3EnvMax, s->m_fEffectiveRadius, s->m_uMaxParticles);
    }
}

template <class S>
static void set_particles(S *s, int n, const float *pos4, const float *vel4) {
    s->m_uNumParticles = (uint)n;
    for (int i = 0; i < n * DIM; ++i) {
        s->m_hPos[i] = pos4[i];
        s->m_hVel[i] = vel4 ? vel4[i] : 0.0f;
    }
}

extern "C" {

/* ---- PBF (rxPBDSPH) ---- */
void *fsph_ref_pbf_create(const fsph_ref_env *e) {
    rxPBDSPH *s = new rxPBDSPH();
    s->Initialize(make_env(e));
    apply_overrides(s, e);
    return s;
}
void fsph_ref_pbf_destroy(void *p) { delete (rxPBDSPH *)p; }
void fsph_ref_pbf_set(void *p, int n, const float *pos4, const float *vel4) {
    set_particles((rxPBDSPH *)p, n, pos4, vel4);
}
int fsph_ref_pbf_update(void *p, float dt, double *eta_out) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    s->Update(dt, 0);
    if (eta_out) *eta_out = g_fEta;
    return g_iIterations;
}
/* which: 0 pos, 1 vel, 2 dens, 3 scaling factor, 4 dp, 5 predicted pos, 6 force */
void fsph_ref_pbf_get(void *p, int which, float *out) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    size_t n4 = (size_t)s->m_uNumParticles * DIM, n1 = s->m_uNumParticles;
    const RXREAL *src = nullptr; size_t cnt = 0;
    switch (which) {
    case 0: src = s->m_hPos; cnt = n4; break;
    case 1: src = s->m_hVel; cnt = n4; break;
    case 2: src = s->m_hDens; cnt = n1; break;
    case 3: src = s->m_hS; cnt = n1; break;
    case 4: src = s->m_hDp; cnt = n4; break;
    case 5: src = s->m_hPredictPos; cnt = n4; break;
    case 6: src = s->m_hFrc; cnt = n4; break;
    default: return;
    }
    for (size_t i = 0; i < cnt; ++i) out[i] = src[i];
}
/* h, particle radius, rest density, mass, Aw, Ag, Al, env min xyz, env max xyz */
void fsph_ref_pbf_scalars(void *p, double *out) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    out[0] = s->m_fEffectiveRadius; out[1] = s->m_fParticleRadius; out[2] = s->m_fRestDens;
    out[3] = s->m_fMass; out[4] = s->m_fAw; out[5] = s->m_fAg; out[6] = s->m_fAl;
    for (int k = 0; k < 3; ++k) { out[7 + k] = s->m_v3EnvMin[k]; out[10 + k] = s->m_v3EnvMax[k]; }
}

/* Neighbour sets through rxPBDSPH::SetParticlesToCell(prts, n, h): CSR with
 * offsets[n+1]; idx / dist2 hold at most cap entries.  Returns the total. */
long long fsph_ref_neighbors(void *p, const float *pos4, int n, int *offsets, int *idx, float *dist2, long long cap) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    set_particles(s, n, pos4, nullptr);
    s->SetParticlesToCell(s->m_hPos, n, s->m_fEffectiveRadius);
    long long t = 0;
    for (int i = 0; i < n; ++i) {
        offsets[i] = (int)t;
        for (const rxNeigh &nb : s->m_vNeighs[i]) {
            if (t < cap) { idx[t] = nb.Idx; if (dist2) dist2[t] = nb.Dist2; }
            ++t;
        }
    }
    offsets[n] = (int)t;
    return t;
}

/* The density field on a lattice (rxPBDSPH::CalImplicitField -> CalColorField,
 * rx_sph_pbd.cpp:2024-2108) of the given particles: node (i, j, k) at
 * minp + (i, j, k) d, out[k nx ny + j nx + i]. */
void fsph_ref_pbf_density_grid(void *p, const float *pos4, int n, const int *nn, const double *minp,
                               const double *d, float *out) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    set_particles(s, n, pos4, nullptr);
    s->m_pNNGrid->SetObjectToCell(s->m_hPos, n);
    int dims[3] = {nn[0], nn[1], nn[2]};
    s->CalImplicitField(dims, Vec3(minp[0], minp[1], minp[2]), Vec3(d[0], d[1], d[2]), out);
}

/* rxNNGrid::CalGridHash(Vec3) of the reference's CPU grid for each position,
 * and the grid's cell count. */
long long fsph_ref_cell_hash(void *p, const float *pos4, int n, unsigned int *out) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    for (int i = 0; i < n; ++i)
        out[i] = s->m_pNNGrid->CalGridHash(Vec3(pos4[4 * i + 0], pos4[4 * i + 1], pos4[4 * i + 2]));
    return (long long)s->m_pNNGrid->GetCellData().uNumCells;
}

/* One lambda pass (rxPBDSPH::calScalingFactor) on the given predicted positions. */
void fsph_ref_pbf_lambda(void *p, const float *pos4, int n, float dt, float *dens, float *scl) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    for (int i = 0; i < n * DIM; ++i) s->m_hPredictPos[i] = pos4[i];
    s->m_uNumParticles = n;
    s->SetParticlesToCell(s->m_hPredictPos, n, s->m_fKernelRadius);
    s->calScalingFactor(s->m_hPredictPos, s->m_hDens, s->m_hS, s->m_fEffectiveRadius, dt);
    for (int i = 0; i < n; ++i) { dens[i] = s->m_hDens[i]; scl[i] = s->m_hS[i]; }
}

/* One position-correction pass (rxPBDSPH::calPositionCorrection). */
void fsph_ref_pbf_dp(void *p, const float *pos4, const float *scl, int n, float dt, float *dp4) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    for (int i = 0; i < n * DIM; ++i) s->m_hPredictPos[i] = pos4[i];
    for (int i = 0; i < n; ++i) s->m_hS[i] = scl[i];
    s->m_uNumParticles = n;
    s->SetParticlesToCell(s->m_hPredictPos, n, s->m_fKernelRadius);
    for (int i = 0; i < n * DIM; ++i) s->m_hDp[i] = 0.0f;
    s->calPositionCorrection(s->m_hPredictPos, s->m_hS, s->m_hDp, s->m_fEffectiveRadius, dt);
    for (int i = 0; i < n * DIM; ++i) dp4[i] = s->m_hDp[i];
}

/* Density + external/viscous force + prediction, i.e. Update up to the loop
 * (rx_sph_pbd.cpp:405-418).  Writes dens, frc(4N), predicted pos/vel (4N). */
void fsph_ref_pbf_predict(void *p, float dt, float *dens, float *frc4, float *ppos4, float *pvel4) {
    rxPBDSPH *s = (rxPBDSPH *)p;
    int n = (int)s->m_uNumParticles;
    for (int i = 0; i < n * DIM; ++i) s->m_hFrc[i] = 0.0f;
    s->SetParticlesToCell();
    s->calDensity(s->m_hPos, s->m_hDens, s->m_fEffectiveRadius);
    s->calForceExtAndVisc(s->m_hPos, s->m_hVel, s->m_hDens, s->m_hFrc, s->m_fEffectiveRadius);
    s->integrate(s->m_hPos, s->m_hVel, s->m_hDens, s->m_hFrc, s->m_hPredictPos, s->m_hPredictVel, dt);
    for (int i = 0; i < n; ++i) dens[i] = s->m_hDens[i];
    for (int i = 0; i < n * DIM; ++i) { frc4[i] = s->m_hFrc[i]; ppos4[i] = s->m_hPredictPos[i]; pvel4[i] = s->m_hPredictVel[i]; }
}

/* ---- WCSPH (rxSPH) ---- */
void *fsph_ref_sph_create(const fsph_ref_env *e) {
    rxSPH *s = new rxSPH();
    s->Initialize(make_env(e));
    apply_overrides(s, e);
    return s;
}
void fsph_ref_sph_destroy(void *p) { delete (rxSPH *)p; }
void fsph_ref_sph_set(void *p, int n, const float *pos4, const float *vel4) {
    set_particles((rxSPH *)p, n, pos4, vel4);
}
void fsph_ref_sph_update(void *p, float dt) { ((rxSPH *)p)->Update(dt, 0); }
/* which: 0 pos, 1 vel, 2 dens, 3 pressure, 4 force */
void fsph_ref_sph_get(void *p, int which, float *out) {
    rxSPH *s = (rxSPH *)p;
    size_t n4 = (size_t)s->m_uNumParticles * DIM, n1 = s->m_uNumParticles;
    const RXREAL *src = nullptr; size_t cnt = 0;
    switch (which) {
    case 0: src = s->m_hPos; cnt = n4; break;
    case 1: src = s->m_hVel; cnt = n4; break;
    case 2: src = s->m_hDens; cnt = n1; break;
    case 3: src = s->m_hPres; cnt = n1; break;
    case 4: src = s->m_hFrc; cnt = n4; break;
    default: return;
    }
    for (size_t i = 0; i < cnt; ++i) out[i] = src[i];
}
void fsph_ref_sph_scalars(void *p, double *out) {
    rxSPH *s = (rxSPH *)p;
    out[0] = s->m_fEffectiveRadius; out[1] = s->m_fParticleRadius; out[2] = s->m_fRestDens;
    out[3] = s->m_fMass; out[4] = s->m_fAw; out[5] = s->m_fAg; out[6] = s->m_fAl;
    for (int k = 0; k < 3; ++k) { out[7 + k] = s->m_v3EnvMin[k]; out[10 + k] = s->m_v3EnvMax[k]; }
}
/* Density and force passes on the current positions (rx_sph_cpu.cpp:343-352). */
void fsph_ref_sph_forces(void *p, float *dens, float *pres, float *frc4) {
    rxSPH *s = (rxSPH *)p;
    int n = (int)s->m_uNumParticles;
    s->SetParticlesToCell();
    s->calDensity(s->m_hPos, s->m_hDens, s->m_fEffectiveRadius);
    s->calForce(s->m_hPos, s->m_hVel, s->m_hDens, s->m_hPres, s->m_hFrc, s->m_fEffectiveRadius);
    for (int i = 0; i < n; ++i) { dens[i] = s->m_hDens[i]; pres[i] = s->m_hPres[i]; }
    for (int i = 0; i < n * DIM; ++i) frc4[i] = s->m_hFrc[i];
}

/* ---- kernel functions (rx_kernel.h) and the box wall (rx_sph_solid.cpp) ---- */
/* which: 0 poly6 W, 1 spiky gradient factor a*q*q/r (the scalar multiplying rij),
 * 2 viscosity Laplacian; the coefficient comes from the matching KernelCoef*. */
double fsph_ref_kernel(int which, double r, double h) {
    switch (which) {
    case 0: return KernelPoly6(r, h, KernelCoefPoly6(h, 3, 1));
    case 1: { Vec3 g = KernelSpikyG<Vec3>(r, h, KernelCoefSpiky(h, 3, 2), Vec3(r, 0.0, 0.0));
              return r > 0.0 ? g[0] / r : 0.0; }
    case 2: return KernelViscL(r, h, KernelCoefVisc(h, 3, 3), 3);
    }
    return 0.0;
}
double fsph_ref_kernel_coef(int which, double h) {
    switch (which) {
    case 0: return KernelCoefPoly6(h, 3, 1);
    case 1: return KernelCoefSpiky(h, 3, 2);
    case 2: return KernelCoefVisc(h, 3, 3);
    }
    return 0.0;
}
/* rxSolidBox(cen-ext, cen+ext, -1).GetDistanceR(pos, r): writes the contact
 * point and returns 1 when the point was projected. */
int fsph_ref_wall(const double *cen, const double *ext, double r, const double *pos, double *out) {
    Vec3 c(cen[0], cen[1], cen[2]), e(ext[0], ext[1], ext[2]);
    rxSolidBox box(c - e, c + e, -1);
    rxCollisionInfo col;
    Vec3 p(pos[0], pos[1], pos[2]);
    bool hit = box.GetDistanceR(p, r, col);
    Vec3 q = hit ? col.Contact() : p;
    out[0] = q[0]; out[1] = q[1]; out[2] = q[2];
    return hit ? 1 : 0;
}

}  /* extern "C" */
