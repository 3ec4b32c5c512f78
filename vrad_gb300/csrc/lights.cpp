// lights.cpp -- direct-light parameters (rad/lightmap/lights.go:210-426,
// vmath/quadratic/solver.go:4-69, vmath/quadratic/lerp.go:14-16).
#include <cmath>

#include "vrg_internal.h"

namespace vrg {

namespace {

constexpr float kEqualEpsilon = 0.001f;  // vmath/constants.go:9

// "a x^2 + b x + c = y" through three points, float32 as in solver.go:48-63.
bool solve_inverse_quadratic(float x1, float y1, float x2, float y2, float x3, float y3, float &a,
                             float &b, float &c) {
    const float det = ((x1 - x2) * (x1 - x3)) * (x2 - x3);
    if (det == 0.0f) return false;
    a = ((x3 * (-y1 + y2) + x2 * (y1 - y3)) + x1 * (-y2 + y3)) / det;
    b = (((x3 * x3) * (y1 - y2) + (x1 * x1) * (y2 - y3)) + (x2 * x2) * (-y1 + y3)) / det;
    c = ((((x1 * x3) * (-x1 + x3)) * y2 + (x2 * x2) * ((x3 * y1) - (x1 * y3))) +
         x2 * (-((x3 * x3) * y1) + (x1 * x1) * y3)) /
        det;
    return true;
}

// solver.go:4-45: blend the middle point toward the chord, 0.05 at a time,
// until the derivative at x1 has the monotone sign.  The points are sorted
// by value (solver.go's vSwap swaps local pointers and sorts nothing).
bool solve_inverse_quadratic_monotonic(float x1, float y1, float x2, float y2, float x3, float y3,
                                       float &a, float &b, float &c) {
    if (x1 > x2) {
        std::swap(x1, x2);
        std::swap(y1, y2);
    }
    if (x2 > x3) {
        std::swap(x2, x3);
        std::swap(y2, y3);
    }
    if (x1 > x2) {
        std::swap(x1, x2);
        std::swap(y1, y2);
    }
    for (double blend = 0.0; blend <= 1.0; blend += 0.05) {
        const double lerp = (double)(y1 + ((y3 - y1) * (x2 - x1)) / (x3 - x1));
        const double ty2 = (1.0 - blend) * (double)y2 + blend * lerp;
        if (!solve_inverse_quadratic(x1, y1, x2, (float)ty2, x3, y3, a, b, c)) return false;
        const float deriv = 2.0f * a + b;
        if (y1 < y2 && y2 < y3) {
            if (deriv >= 0.0f) return true;
        } else if (y1 > y2 && y2 > y3) {
            if (deriv <= 0.0f) return true;
        } else {
            return true;
        }
    }
    return true;
}

}  // namespace

// SetLightFalloffParams (lights.go:259-341)
void light_set_falloff(const vrg_light_keys &k, vrg_light &l) {
    const float d50 = k.fifty_percent_distance;
    l.start_fade = 0.0f;
    l.end_fade = -1.0f;
    l.cap_distance = 1.0e22f;
    if (d50 != 0.0f) {
        float d0 = k.zero_percent_distance;
        if (d0 < d50) d0 = 2.0f * d50;
        float a = 0.0f, b = 1.0f, c = 0.0f;
        solve_inverse_quadratic_monotonic(0.0f, 1.0f, d50, 2.0f, d0, 256.0f, a, b, c);
        const float v50 = c + d50 * (b + d50 * a);
        const float scale = 2.0f / v50;
        a *= scale;
        b *= scale;
        c *= scale;
        l.quadratic_attn = a;
        l.linear_attn = b;
        l.constant_attn = c;
        if (k.hard_falloff != 0) {
            l.end_fade = d0;
            l.start_fade = 0.75f * d0 + 0.25f * d50;
        } else if (std::fabs((double)a) > 0.0) {
            const float fmax = b / (-2.0f * a);
            if (fmax > 0.0f) {
                l.cap_distance = fmax;
                l.start_fade = fmax;
                l.end_fade = 10.0f * fmax;
            }
        }
        return;
    }
    l.constant_attn = k.constant_attn;
    l.linear_attn = k.linear_attn;
    l.quadratic_attn = k.quadratic_attn;
    l.radius = k.distance;
    if (l.constant_attn < kEqualEpsilon) l.constant_attn = 0.0f;
    if (l.linear_attn < kEqualEpsilon) l.linear_attn = 0.0f;
    if (l.quadratic_attn < kEqualEpsilon) l.quadratic_attn = 0.0f;
    if (l.constant_attn < kEqualEpsilon && l.linear_attn < kEqualEpsilon &&
        l.quadratic_attn < kEqualEpsilon)
        l.constant_attn = 1.0f;
    // scale intensity for unit 100 distance
    const float ratio = (l.constant_attn + 100.0f * l.linear_attn) + 10000.0f * l.quadratic_attn;
    if (ratio > 0.0f)
        for (float &i : l.intensity) i = i * ratio;
}

// ParseLightSpot (lights.go:210-257), cone keys only
void light_parse_spot(const vrg_light_keys &k, vrg_light &l) {
    const float pi = (float)3.14159265358979323846;
    l.type = VRG_EMIT_SPOTLIGHT;
    l.stopdot = k.inner_cone == 0.0f ? 10.0f : k.inner_cone;
    l.stopdot2 = k.cone == 0.0f ? l.stopdot : k.cone;
    if (l.stopdot2 < l.stopdot) l.stopdot2 = l.stopdot;
    if (l.stopdot == 180.0f && l.stopdot2 == 180.0f) {
        l.stopdot = 0.0f;
        l.stopdot2 = 0.0f;
        l.type = VRG_EMIT_POINT;
        l.exponent = 0.0f;
    } else {
        // clamp to 90 degrees (lights.go:238-249)
        l.stopdot = std::min(l.stopdot, 90.0f);
        l.stopdot2 = std::min(l.stopdot2, 90.0f);
        l.stopdot2 = (float)std::cos((double)((l.stopdot2 / 180.0f) * pi));
        l.stopdot = (float)std::cos((double)((l.stopdot / 180.0f) * pi));
        l.exponent = k.exponent;
    }
    light_set_falloff(k, l);
}

}  // namespace vrg
