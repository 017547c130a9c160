/*
 * Test-infrastructure class declarations for the oracle/_ref translation unit.
 *
 * The reference declares rxSolid / rxSolidBox (rx_sph_solid.h:83-187) and
 * rxSPH / rxPBDSPH (rx_sph.h:202-426, 1027-1274) next to GL, VBO and boost
 * members.  These declarations carry only the members that the reference's
 * own CPU fluid functions (extracted by extract.py) read and write, with the
 * same names and types, so that those function bodies compile unchanged.
 * Members that only matter for drawing, turbulence, anisotropic kernels or
 * ice coupling are left out.  Rotation is the identity for the domain box, as
 * in rxSolid's constructor (rx_sph_solid.h:97-106).
 */
#ifndef FSPH_REF_HARNESS_CLASSES_H
#define FSPH_REF_HARNESS_CLASSES_H

class rxSolid {
public:
    Vec3 m_vMassCenter;
    Vec3 m_vVelocity;
    int m_iSgn;
    rxSolid() : m_vMassCenter(0.0), m_vVelocity(0.0), m_iSgn(1) {}
    virtual ~rxSolid() {}
    virtual bool GetDistanceR(const Vec3 &pos, const double &r, rxCollisionInfo &col) = 0;
    virtual Vec3 GetMin(void) = 0;
    virtual Vec3 GetMax(void) = 0;
    /* Identity-rotation form of rxSolid::CalLocalCoord (rx_sph_solid.h:272-282). */
    Vec3 CalLocalCoord(const Vec3 &pos) { return pos - m_vMassCenter; }
    Vec3 GetVelocityAtGrobal(const Vec3 &) { return m_vVelocity; }
};

class rxSolidBox : public rxSolid {
public:
    Vec3 m_vMax, m_vMin;
    /* Same construction as rx_sph_solid.h:167-177. */
    rxSolidBox(Vec3 minp, Vec3 maxp, int sgn) {
        Vec3 sl = 0.5 * (maxp - minp);
        Vec3 ctr = 0.5 * (maxp + minp);
        m_vMin = -sl;
        m_vMax = sl;
        m_vMassCenter = ctr;
        m_iSgn = sgn;
    }
    Vec3 GetMin(void) { return m_vMassCenter + m_vMin; }
    Vec3 GetMax(void) { return m_vMassCenter + m_vMax; }
    bool GetDistanceR(const Vec3 &pos, const double &r, rxCollisionInfo &col);
};

/* Members shared by both solvers (rxParticleSystemBase, rx_ps.h:119-190). */
class fsphRefBase {
public:
    bool m_bInitialized = false;
    uint m_uNumParticles = 0;
    uint m_uMaxParticles = 0;
    uint m_uNumBParticles = 0;
    RXREAL m_fParticleRadius = 0.1f;
    Vec3 m_v3Gravity = Vec3(0.0, -9.82, 0.0);
    RXREAL m_fDamping = 0.0f;
    RXREAL m_fRestitution = 0.0f;
    RXREAL *m_hPos = nullptr;
    RXREAL *m_hVel = nullptr;
    Vec3 m_v3EnvMin, m_v3EnvMax;
    int m_iColorType = 0;
    vector<rxInletLine> m_vInletLines;
    int m_iInletStart = -1;

    float GetParticleRadius() { return m_fParticleRadius; }
    void SetGravity(RXREAL x) { m_v3Gravity = Vec3(0.0, x, 0.0); }
    /* Host copies are the state on the CPU path; VBO upload and colouring are GUI-only. */
    void SetArrayVBO(rxParticleArray, const RXREAL *, int, int) {}
    void SetColorVBO(int) {}
    int addParticles(int &, rxInletLine, int = 0) { return 0; }
};

class rxPBDSPH : public fsphRefBase {
public:
    RXREAL *m_hNrm = nullptr, *m_hFrc = nullptr, *m_hDens = nullptr, *m_hPres = nullptr;
    RXREAL *m_hS = nullptr, *m_hDp = nullptr;
    RXREAL *m_hPredictPos = nullptr, *m_hPredictVel = nullptr;
    rxSolid *m_pBoundary = nullptr;
    vector<rxSolid *> m_vSolids;
    int m_iNumTris = 0;
    rxNNGrid *m_pNNGrid = nullptr;
    vector<vector<rxNeigh> > m_vNeighs;
    uint m_iKernelParticles = 0;
    RXREAL m_fRestDens = 0, m_fMass = 0;
    RXREAL m_fEffectiveRadius = 0;
    RXREAL m_fKernelRadius = 0;
    RXREAL m_fGasStiffness = 1.0f;
    RXREAL m_fViscosity = 0.0f;
    RXREAL m_fEpsilon = 0.01f;
    RXREAL m_fEta = 0.05f;
    int m_iMinIterations = 2;
    int m_iMaxIterations = 10;
    bool m_bArtificialPressure = true;
    RXREAL m_fApK = 0.1f, m_fApN = 4.0f, m_fApQ = 0.2f;
    double m_fAw = 0, m_fAg = 0, m_fAl = 0;
    double (*m_fpW)(double, double, double) = nullptr;
    Vec3 (*m_fpGW)(double, double, double, Vec3) = nullptr;
    double (*m_fpLW)(double, double, double, double) = nullptr;

    rxPBDSPH() { m_pNNGrid = new rxNNGrid(DIM); }
    ~rxPBDSPH();
    void Initialize(const rxSPHEnviroment &env);
    void Allocate(int max_particles);
    bool Update(RXREAL dt, int step = 0);
    void calDensity(const RXREAL *pos, RXREAL *dens, RXREAL h);
    void calForceExtAndVisc(const RXREAL *pos, const RXREAL *vel, const RXREAL *dens, RXREAL *frc, RXREAL h);
    void calScalingFactor(const RXREAL *ppos, RXREAL *pdens, RXREAL *pscl, RXREAL h, RXREAL dt);
    void calPositionCorrection(const RXREAL *ppos, const RXREAL *pscl, RXREAL *pdp, RXREAL h, RXREAL dt);
    RXREAL calRestDensity(RXREAL h);
    void integrate(const RXREAL *pos, const RXREAL *vel, const RXREAL *dens, const RXREAL *acc,
                   RXREAL *pos_new, RXREAL *vel_new, RXREAL dt);
    int calCollisionPolygon(uint, Vec3 &, Vec3 &, Vec3 &, RXREAL) { return 0; }
    int calCollisionSolid(Vec3 &pos0, Vec3 &pos1, Vec3 &vel, RXREAL dt);
    void GetNearestNeighbors(Vec3 pos, vector<rxNeigh> &neighs, RXREAL h = -1.0);
    void GetNearestNeighbors(int idx, RXREAL *p, vector<rxNeigh> &neighs, RXREAL h = -1.0);
    void SetParticlesToCell(void);
    void SetParticlesToCell(RXREAL *prts, int n, RXREAL h);
    double GetImplicit(double x, double y, double z);
    void CalImplicitField(int n[3], Vec3 minp, Vec3 d, RXREAL *hF);
    double CalColorField(double x, double y, double z);
};

class rxSPH : public fsphRefBase {
public:
    RXREAL *m_hNrm = nullptr, *m_hFrc = nullptr, *m_hDens = nullptr, *m_hPres = nullptr;
    rxSolid *m_pBoundary = nullptr;
    vector<rxSolid *> m_vSolids;
    int m_iNumTris = 0;
    rxNNGrid *m_pNNGrid = nullptr;
    vector<vector<rxNeigh> > m_vNeighs;
    uint m_iKernelParticles = 0;
    RXREAL m_fRestDens = 0, m_fMass = 0;
    RXREAL m_fEffectiveRadius = 0;
    /* rxSPH::Initialize never assigns it before calRestDensity reads it
     * (rx_sph_cpu.cpp:710); the harness starts it at 0 so the read is defined. */
    RXREAL m_fKernelRadius = 0;
    RXREAL m_fGasStiffness = 3.0f;
    RXREAL m_fViscosity = 0.0f;
    double m_fAw = 0, m_fAg = 0, m_fAl = 0;
    double (*m_fpW)(double, double, double) = nullptr;
    Vec3 (*m_fpGW)(double, double, double, Vec3) = nullptr;
    double (*m_fpLW)(double, double, double, double) = nullptr;

    rxSPH() { m_pNNGrid = new rxNNGrid(DIM); }
    ~rxSPH();
    void Initialize(const rxSPHEnviroment &env);
    void Allocate(int max_particles);
    bool Update(RXREAL dt, int step = 0);
    void calDensity(const RXREAL *pos, RXREAL *dens, RXREAL h);
    void calForce(const RXREAL *ppos, const RXREAL *pvel, const RXREAL *pdens, RXREAL *ppres, RXREAL *pfrc, RXREAL h);
    RXREAL calRestDensity(RXREAL h);
    void integrate(const RXREAL *pos, const RXREAL *vel, const RXREAL *dens, const RXREAL *acc,
                   RXREAL *pos_new, RXREAL *vel_new, RXREAL dt);
    int calCollisionPolygon(uint, Vec3 &, Vec3 &, Vec3 &, RXREAL) { return 0; }
    int calCollisionSolid(Vec3 &pos0, Vec3 &pos1, Vec3 &vel, RXREAL dt);
    void GetNearestNeighbors(Vec3 pos, vector<rxNeigh> &neighs, RXREAL h = -1.0);
    void GetNearestNeighbors(int idx, RXREAL *p, vector<rxNeigh> &neighs, RXREAL h = -1.0);
    void SetParticlesToCell(void);
    void SetParticlesToCell(RXREAL *prts, int n, RXREAL h);
};

#endif
