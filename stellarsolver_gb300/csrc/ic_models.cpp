// Initial conditions reproducing the reference's generators draw for draw
// (BarnesHutParticleSystem.cpp:390-560).  The expressions keep the reference's
// operand types (float draws, double literals and <math.h> overloads), because
// they decide the rounding of every position and velocity.
#include "ic_models.h"
#include "stellar_bh.h"

#include <math.h>

#include <random>
#include <vector>

namespace ssg_ic {

namespace {
const float kPi = 3.14159265;  // the reference's constant (BarnesHutParticleSystem.cpp:393)
}

void plummer(float* mass, float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n) {
    const float a = 1.0;
    std::default_random_engine gen;
    std::uniform_real_distribution<float> unit(0, 1.0);
    std::uniform_real_distribution<float> tenth(0, 0.1);
    std::uniform_real_distribution<float> angle(0.0, 2 * kPi);
    std::uniform_real_distribution<float> cosine(-1.0, 1.0);
    for (int i = 0; i < n; i++) {
        float phi = angle(gen);
        float polar = acos(cosine(gen));  // drawn and unused, as in the reference
        (void)polar;
        float r = a / sqrt(pow(unit(gen), -0.666666) - 1);
        mass[i] = 1.0;
        x[i] = r * cos(phi);
        y[i] = r * sin(phi);
        float s = 0.0;
        float t = 0.1;
        while (t > s * s * pow(1.0 - s * s, 3.5)) {
            s = unit(gen);
            t = tenth(gen);
        }
        float v = 100 * s * sqrt(2) * pow(1.0 + r * r, -0.25);
        phi = angle(gen);
        polar = acos(cosine(gen));
        vx[i] = v * cos(phi);
        vy[i] = v * sin(phi);
        ax[i] = 0.0;
        ay[i] = 0.0;
    }
}

void disk(float* mass, float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n,
          float gravity) {
    std::default_random_engine gen;
    std::uniform_real_distribution<float> radius(1.5, 12.0);
    std::uniform_real_distribution<float> angle(0.0, 2 * kPi);
    for (int i = 0; i < n; i++) {
        float theta = angle(gen);
        float r = radius(gen);
        if (i == 0) {
            mass[i] = 200000;
            x[i] = 0;
            y[i] = 0;
        } else {
            mass[i] = 1.0;
            x[i] = r * cos(theta);
            y[i] = r * sin(theta);
        }
        float rotation = -1;  // counter-clockwise
        float v = 1.0 * sqrt(gravity * 200000.0 / r);
        if (i == 0) {
            vx[0] = 0;
            vy[0] = 0;
        } else {
            vx[i] = rotation * v * sin(theta);
            vy[i] = -rotation * v * cos(theta);
        }
        ax[i] = 0.0;
        ay[i] = 0.0;
    }
}

void colliding_disks(float* mass, float* x, float* y, float* vx, float* vy, float* ax, float* ay,
                     int n, float gravity) {
    std::default_random_engine gen;
    std::uniform_real_distribution<float> radius1(1.5, 12.0);
    std::uniform_real_distribution<float> radius2(1, 5.0);
    std::uniform_real_distribution<float> angle(0.0, 2 * kPi);
    for (int i = 0; i < n; i++) {
        float theta = angle(gen);
        float r1 = radius1(gen);
        float r2 = radius2(gen);
        if (i == 0) {
            mass[i] = 100000;
            x[i] = 0;
            y[i] = 0;
        } else if (i == 1) {
            mass[i] = 25000;
            x[i] = 20 * cos(theta);
            y[i] = 20 * sin(theta);
        } else if (i <= 3 * n / 4) {
            mass[i] = 1.0;
            x[i] = r1 * cos(theta);
            y[i] = r1 * sin(theta);
        } else {
            mass[i] = 1.0;
            x[i] = r2 * cos(theta) + x[1];
            y[i] = r2 * sin(theta) + y[1];
        }
        float rotation = 1;  // clockwise
        float v1 = 1.0 * sqrt(gravity * 100000.0 / r1);
        float v2 = 1.0 * sqrt(gravity * 25000.0 / r2);
        if (i == 0 || i == 1) {
            vx[i] = 0.0;
            vy[i] = 0.0;
        } else if (i <= 3 * n / 4) {
            vx[i] = rotation * v1 * sin(theta);
            vy[i] = -rotation * v1 * cos(theta);
        } else {
            vx[i] = rotation * v2 * sin(theta);
            vy[i] = -rotation * v2 * cos(theta);
        }
        ax[i] = 0.0;
        ay[i] = 0.0;
    }
}

}  // namespace ssg_ic

extern "C" int bh_initial_conditions(int model, int n, float gravity, float* mass, float* x,
                                     float* y, float* vx, float* vy) {
    if (n < 1 || !mass || !x || !y || !vx || !vy) return BH_ERR_ARG;
    std::vector<float> ax(n), ay(n);
    switch (model) {
        case BH_MODEL_DISK: ssg_ic::disk(mass, x, y, vx, vy, ax.data(), ay.data(), n, gravity); break;
        case BH_MODEL_COLLIDING_DISKS:
            ssg_ic::colliding_disks(mass, x, y, vx, vy, ax.data(), ay.data(), n, gravity);
            break;
        case BH_MODEL_PLUMMER: ssg_ic::plummer(mass, x, y, vx, vy, ax.data(), ay.data(), n); break;
        default: return BH_ERR_ARG;
    }
    return BH_OK;
}
