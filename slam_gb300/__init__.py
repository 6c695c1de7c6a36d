"""slam_gb300: GB300-native dense RGB-D tracking (the frame-to-model
ICP + photometric odometry step of siw-engineering/slam / ElasticFusion).

The product is the native library libslam_gb300.so (C ABI declared in
include/slam_gb300.h); this package builds it in-tree and mirrors the
reference's RGBDOdometryef interface in Python for tests and benchmarks.
"""
from .odometry import (RGBDOdometry, OdometryError, MODE_GRAPH, MODE_STREAM, MODE_PERSISTENT, PREC_FP32,
                       PREC_COMPENSATED, DEFAULT_ANGLE_THRESH, DEFAULT_DIST_THRESH)

__all__ = ["RGBDOdometry", "OdometryError", "MODE_GRAPH", "MODE_STREAM", "MODE_PERSISTENT", "PREC_FP32",
           "PREC_COMPENSATED", "DEFAULT_ANGLE_THRESH", "DEFAULT_DIST_THRESH"]
