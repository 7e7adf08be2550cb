// Build shim: the minimal declarations that let the reference's own
// Source/SceneManager.cpp compile here without glm, Qt or the Banana library.
// It declares the same class interface as the reference's
// Include/SceneManager.h:25-38 and a vector type with glm::vec3's per-component
// float arithmetic; it contains no scene logic.  Used only by build_ref.sh
// (also by the Simulator shim beside it).
#pragma once
#include <cmath>
#include <memory>
#include <vector>

template <typename T>
struct Vec3 {
    T v[3];
    Vec3() : v{T(0), T(0), T(0)} {}
    template <typename U>
    explicit Vec3(U s) : v{static_cast<T>(s), static_cast<T>(s), static_cast<T>(s)} {}
    template <typename A, typename B, typename C>
    Vec3(A a, B b, C c) : v{static_cast<T>(a), static_cast<T>(b), static_cast<T>(c)} {}
    T& operator[](int i) { return v[i]; }
    const T& operator[](int i) const { return v[i]; }
    Vec3& operator+=(const Vec3& o) {
        for (int i = 0; i < 3; ++i) v[i] = v[i] + o.v[i];
        return *this;
    }
};
template <typename T>
Vec3<T> operator+(const Vec3<T>& a, const Vec3<T>& b) { return Vec3<T>(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
template <typename T>
Vec3<T> operator-(const Vec3<T>& a, const Vec3<T>& b) { return Vec3<T>(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
template <typename T>
Vec3<T> operator*(T s, const Vec3<T>& a) { return Vec3<T>(s * a[0], s * a[1], s * a[2]); }
template <typename T>
Vec3<T> operator*(const Vec3<T>& a, T s) { return Vec3<T>(a[0] * s, a[1] * s, a[2] * s); }
template <typename T>
using Vec_Vec3 = std::vector<Vec3<T>>;

namespace glm {
// glm::length(vec3) = sqrt(dot(v, v)) with dot = (x*x + y*y) + z*z
inline float length(const Vec3<float>& a) { return std::sqrt((a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]); }
}  // namespace glm

class SimulationScenes {
public:
    enum Scene { SphereDrop = 0, CubeDrop, Dambreak, DoubleDambreak };
};

template <typename T>
struct SPHParameters {
    T particleRadius = T(0);
    int scene = 0;
    int numThreads = 0;  // read by Source/Simulator.cpp
    T stopTime = T(5);
};

class SceneManager {
public:
    SceneManager(std::shared_ptr<SPHParameters<float> >& simParams) : m_SimParams(simParams) {}
    void setupScene(Vec_Vec3<float>& particles, Vec_Vec3<float>& velocity);
    void setupSceneCubeDrop(Vec_Vec3<float>& particles, Vec_Vec3<float>& velocity);
    void setupSceneSphereDrop(Vec_Vec3<float>& particles, Vec_Vec3<float>& velocity);
    void setupSceneDambreak(Vec_Vec3<float>& particles, Vec_Vec3<float>& velocity);
    void setupSceneDoubleDambreak(Vec_Vec3<float>& particles, Vec_Vec3<float>& velocity);

private:
    std::shared_ptr<SPHParameters<float> >& m_SimParams;
};
