"""GB300-native GWRBasic engine (drop-in for libgwmodel's gwm::GWRBasic).

The compute path is libgwgpu.so: hand-written sm_103a CUDA kernels behind a
C ABI (include/gwgpu.h).  This package is its Python face.
"""
from .gwrbasic import (BandwidthWeight, CRSDistance, Engine, GwgpuError, GWRBasic, LogLevel, Logger,
                       ParallelType, Precision, RegressionDiagnostic, SpatialWeight, Status)
from .mgwr import GWRMultiscale

__all__ = ["GWRBasic", "GWRMultiscale", "CRSDistance", "BandwidthWeight", "SpatialWeight", "RegressionDiagnostic", "Logger",
           "ParallelType", "Status", "Precision", "LogLevel", "Engine", "GwgpuError"]
