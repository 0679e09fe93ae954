// Headless stand-in for openFrameworks' ofMain.h, written for this project.
//
// TEST INFRASTRUCTURE ONLY. It lets the reference's own hot-path translation units
// (src/{MathUtils,Body,OctantUtils,HashedNode,HashedOctree}.cpp) compile without
// openFrameworks so they can serve as the REF-LITERAL oracle. Nothing on the
// arithmetic path depends on openFrameworks: ofColor is display-only, and the draw
// calls used by the visualisation helpers become no-ops here.
#pragma once
#include <bitset>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <random>
#include <stack>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>
using namespace std;

#ifndef PI
#define PI 3.14159265358979323846
#endif

struct ofColor {
  unsigned char r = 0, g = 0, b = 0, a = 255;
  ofColor() {}
  ofColor(int R, int G, int B, int A = 255)
      : r((unsigned char)R), g((unsigned char)G), b((unsigned char)B), a((unsigned char)A) {}
};

inline float ofGetElapsedTimef() {
  static const auto t0 = std::chrono::steady_clock::now();
  return std::chrono::duration<float>(std::chrono::steady_clock::now() - t0).count();
}
inline void ofFill() {}
inline void ofNoFill() {}
template <class... A> inline void ofSetColor(A...) {}
template <class... A> inline void ofDrawIcoSphere(A...) {}
template <class... A> inline void ofDrawBox(A...) {}
// A harness may install the generator behind ofRandom (the scene harness installs a
// counter-based one so that the reference's set-up draws known numbers); by default rand().
inline float (*&of_random_unit_hook())() {
  static float (*hook)() = nullptr;
  return hook;
}
inline float of_random_unit() {
  return of_random_unit_hook() ? of_random_unit_hook()() : (float)std::rand() / (float)RAND_MAX;
}
inline float ofRandom(float hi) { return hi * of_random_unit(); }
inline float ofRandom(float lo, float hi) { return lo + (hi - lo) * of_random_unit(); }
inline float ofDegToRad(float deg) { return deg * (float)(PI / 180.0); }
