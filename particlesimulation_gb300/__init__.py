"""GB300-native PM / P3M force-and-step path (CUDA sm_103a behind the C ABI of include/pmgb.h)."""
from .methods import (CloudShape, DiskSamplerLinear, FFTAdapter, FiniteDiffScheme, GreensFunction,
                      InterpolationScheme, LearnedClosure, P3MMethod, PlummerSampler, PMMethod,
                      SphRadDecrField, StateRecorder, setHalfStepVelocities,
                      setIntegerStepVelocities, updatePositions, updateVelocities)

__all__ = ["PMMethod", "P3MMethod", "LearnedClosure", "StateRecorder", "PlummerSampler",
           "DiskSamplerLinear", "InterpolationScheme", "FiniteDiffScheme", "GreensFunction",
           "CloudShape", "SphRadDecrField", "FFTAdapter", "setHalfStepVelocities",
           "setIntegerStepVelocities", "updatePositions", "updateVelocities"]
