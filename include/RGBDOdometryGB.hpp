// Header-only C++ shim over the C ABI (slam_gb300.h) that keeps the method
// names, argument meaning and public statistics of the reference class
// RGBDOdometryef (src/odom/RGBDOdometryef.h:28-131), so existing call sites
// (src/apps/elastic_fusion_file.cpp:367-374, src/model/Model.cpp:318-334,
// src/lc/Ferns.cpp:253-268) keep their shape.  Differences:
//  - textures become device pointers + row pitches (see slam_gb300.h);
//  - poses are plain float arrays (row-major 3x3 rotation, 3-vector
//    translation, row-major 4x4 model pose) instead of Eigen types;
//  - failures throw RGBDOdometryGB::Error instead of exiting the process.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "slam_gb300.h"

class RGBDOdometryGB {
  public:
    struct Error : std::runtime_error {
        int status;
        Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
    };

    RGBDOdometryGB(int width, int height, float cx, float cy, float fx, float fy,
                   float distThresh = ODO_DEFAULT_DIST_THRESH, float angleThresh = ODO_DEFAULT_ANGLE_THRESH) {
        check(odo_create(width, height, cx, cy, fx, fy, distThresh, angleThresh, &h_), "odo_create");
    }
    ~RGBDOdometryGB() { odo_destroy(h_); }
    RGBDOdometryGB(const RGBDOdometryGB &) = delete;
    RGBDOdometryGB &operator=(const RGBDOdometryGB &) = delete;

    void setStream(void *cudaStream) { check(odo_set_stream(h_, cudaStream), "odo_set_stream"); }

    void initICP(const uint16_t *filteredDepth, size_t pitch, const float depthCutoff) {
        check(odo_init_icp_depth(h_, filteredDepth, pitch, depthCutoff), "initICP");
    }
    void initICP(const float *predictedVertices, const float *predictedNormals, size_t pitch,
                 const float depthCutoff) {
        check(odo_init_icp_maps(h_, predictedVertices, predictedNormals, pitch, depthCutoff), "initICP");
    }
    void initICPModel(const float *predictedVertices, const float *predictedNormals, size_t pitch,
                      const float depthCutoff, const float modelPose[16]) {
        check(odo_init_icp_model(h_, predictedVertices, predictedNormals, pitch, depthCutoff, modelPose),
              "initICPModel");
    }
    void initRGB(const uint8_t *rgba, size_t pitch) { check(odo_init_rgb(h_, rgba, pitch), "initRGB"); }
    void initRGBModel(const uint8_t *rgba, size_t pitch) { check(odo_init_rgb_model(h_, rgba, pitch), "initRGBModel"); }
    void initFirstRGB(const uint8_t *rgba, size_t pitch) { check(odo_init_first_rgb(h_, rgba, pitch), "initFirstRGB"); }

    // trans[3], rot[9] (row-major): previous pose in, tracked pose out.
    void getIncrementalTransformation(float trans[3], float rot[9], const bool &rgbOnly, const float &icpWeight,
                                      const bool &pyramid, const bool &fastOdom, const bool &so3) {
        check(odo_get_incremental_transformation(h_, trans, rot, rgbOnly, icpWeight, pyramid, fastOdom, so3),
              "getIncrementalTransformation");
        odo_stats s;
        check(odo_get_stats(h_, &s), "odo_get_stats");
        lastICPError = s.lastICPError;
        lastICPCount = s.lastICPCount;
        lastRGBError = s.lastRGBError;
        lastRGBCount = s.lastRGBCount;
        lastSO3Error = s.lastSO3Error;
        lastSO3Count = s.lastSO3Count;
        for (int i = 0; i < 36; ++i) lastA[i] = s.lastA[i];
        for (int i = 0; i < 6; ++i) lastb[i] = s.lastb[i];
    }

    // Row-major 6x6 inverse of lastA.
    void getCovariance(double out[36]) { check(odo_get_covariance(h_, out), "getCovariance"); }

    float lastICPError = 0, lastICPCount = 0, lastRGBError = 0, lastRGBCount = 0, lastSO3Error = 0,
          lastSO3Count = 0;
    double lastA[36] = {0};
    double lastb[6] = {0};

    odo_t *handle() const { return h_; }

  private:
    void check(int rc, const char *what) {
        if (rc != ODO_OK) throw Error(rc, std::string(what) + ": " + odo_status_string(rc) + " " + odo_last_error(h_));
    }
    odo_t *h_ = nullptr;
};
