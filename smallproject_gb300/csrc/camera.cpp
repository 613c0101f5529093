// camera.cpp - camera matrix and frame constants. Built with -ffp-contract=off so every
// float op rounds separately, in the order the reference host code writes it.
#include "camera.hpp"

#include <cmath>

namespace vxr {

namespace {
struct V3 {
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// precomp.h:684
inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
// precomp.h:283,656: v * (1 / sqrt(dot(v, v)))
inline V3 normalize(V3 v) {
    const float inv = 1.0f / std::sqrt(dot(v, v));
    return v * inv;
}
inline V3 load(const float p[3]) { return v3(p[0], p[1], p[2]); }
inline void store(float p[3], V3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
// TransformPosition (template.cpp:1059-1062) = (M * (a, 1)).xyz (template.cpp:1045-1051)
inline V3 transform_position(V3 a, const Mat4& M) {
    const float* c = M.cell;
    return v3(c[0] * a.x + c[1] * a.y + c[2] * a.z + c[3] * 1.0f, c[4] * a.x + c[5] * a.y + c[6] * a.z + c[7] * 1.0f,
              c[8] * a.x + c[9] * a.y + c[10] * a.z + c[11] * 1.0f);
}
inline void plane(float out[4], V3 n, V3 E) {
    out[0] = n.x; out[1] = n.y; out[2] = n.z;
    out[3] = dot(E, n);
}
// RandomUInt (template.cpp:933-941)
inline uint32_t xorshift(uint32_t& s) {
    s ^= s << 13;
    s ^= s >> 17;
    s ^= s << 5;
    return s;
}
}  // namespace

Mat4 look_at(const float Pp[3], const float Tp[3]) {
    const V3 P = load(Pp), T = load(Tp);
    const V3 z = normalize(T - P);
    const V3 x = normalize(cross(z, v3(0, 1, 0)));
    const V3 y = cross(x, z);
    Mat4 M;
    M.cell[3] = P.x; M.cell[7] = P.y; M.cell[11] = P.z;     // mat4::Translate (precomp.h:869)
    M.cell[0] = x.x; M.cell[4] = x.y; M.cell[8] = x.z;
    M.cell[1] = y.x; M.cell[5] = y.y; M.cell[9] = y.z;
    M.cell[2] = z.x; M.cell[6] = z.y; M.cell[10] = z.z;
    return M;
}

void begin_frame(CameraState& st, uint32_t W, uint32_t H, vxr_frame_consts* k) {
    // backup previous frame data (world.cpp:2144-2149)
    V3 prevE = load(st.E), prevP0 = load(st.p0), prevP1 = load(st.p1), prevP2 = load(st.p2);
    const V3 prevP3 = prevP1 + (prevP2 - prevP0);
    const float aspect = (float)W / (float)H;
    const V3 E = transform_position(v3(0, 0, 0), st.M);
    const V3 p0 = transform_position(v3(aspect, 1, 2.2f), st.M);
    const V3 p1 = transform_position(v3(-aspect, 1, 2.2f), st.M);
    const V3 p2 = transform_position(v3(aspect, -1, 2.2f), st.M);
    if (st.firstFrame) {
        // world.cpp:2160-2166; prevP3 keeps the value computed before (zero corners)
        prevE = E; prevP0 = p0; prevP1 = p1; prevP2 = p2;
        st.firstFrame = false;
    }
    store(st.E, E); store(st.p0, p0); store(st.p1, p1); store(st.p2, p2);
    store(k->E, E); store(k->p0, p0); store(k->p1, p1); store(k->p2, p2);
    k->oneOverRes[0] = 1.0f / (float)W;
    k->oneOverRes[1] = 1.0f / (float)H;
    // previous-frame frustum planes (world.cpp:2167-2175)
    plane(k->Nleft, normalize(cross(prevP0 - prevE, prevP2 - prevE)), prevE);
    plane(k->Nright, normalize(cross(prevP3 - prevE, prevP1 - prevE)), prevE);
    plane(k->Ntop, normalize(cross(prevP0 - prevE, prevP1 - prevE)), prevE);
    plane(k->Nbottom, normalize(cross(prevP3 - prevE, prevP2 - prevE)), prevE);
    k->R0 = xorshift(st.rng);                                   // world.cpp:2184
    k->frame = st.frame;
    k->framecount = st.framecount;
    k->restirtemporalframe = st.restirtemporalframe;
    k->width = W;
    k->height = H;
}

void end_frame(CameraState& st) {
    st.frame = (st.frame + 1) & 255u;
    st.framecount = st.framecount + 1;
    st.restirtemporalframe = st.restirtemporalframe + 1;
}

}  // namespace vxr
