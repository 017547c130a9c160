/*
 * Test-infrastructure prelude for the oracle/_ref translation unit (see
 * extract.py).  Provides the few names the reference's CPU fluid functions
 * take from headers that are either missing from the reference tree or tied
 * to its GUI (timers, console tee, particle-array enum, globals).
 */
#ifndef FSPH_REF_HARNESS_PRELUDE_H
#define FSPH_REF_HARNESS_PRELUDE_H

#include "rx_utility.h"
#include <ostream>

typedef unsigned int uint;

#ifndef DIM
#define DIM 4
#endif

/* A sink for the reference's console output (RXCOUT is a boost tee in
 * rx_sph_commons.h:337-369; the grid setup prints with cout). */
static std::ostream fsph_ref_null_stream(nullptr);
#define RXCOUT fsph_ref_null_stream

/* RXTIMER splits (rx_sph.h:40-58) are GUI instrumentation. */
#define RXTIMER(x)

/* Iteration count and final density error of the last PBF step
 * (rx_sph_pbd.cpp:21-22). */
int g_iIterations = 0;
double g_fEta = 0.0;

/* Particle-array identifiers used by Update's SetArrayVBO calls (rx_ps.h:68-116). */
enum rxParticleArray {
    RX_POSITION = 0, RX_VELOCITY, RX_NORMAL, RX_FORCE, RX_DENSITY, RX_PRESSURE,
    RX_SURFACE, RX_ATTRIBUTE, RX_PREDICT_POS, RX_PREDICT_VEL, RX_SCALING_FACTOR, RX_CORRECTION
};

/* Inlet line (rx_ps.h:39-47); the harness never adds inlets. */
struct rxInletLine {
    Vec3 pos1, pos2, vel, up;
    int accum, span;
    double spacing;
};

#endif
