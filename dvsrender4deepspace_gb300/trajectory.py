"""Analytic camera trajectories for the synthetic workloads.

Each trajectory returns the OpticalState of a time (position, linear
velocity, rotation quaternion, world light direction, intensity and their
rates), i.e. what to_optical_state(CameraTrajectory::evaluate(t)) hands to
the sensor in the reference (include/dvs/raycast.hpp:17-22).  The camera
follows the Blender convention of the reference bundles: it looks along its
local -Z, so the identity rotation looks straight down at the terrain.
"""
import math

import numpy as np


def sun_direction(elevation_deg, azimuth_deg=0.0):
    """Unit vector toward the sun; azimuth 0 is +x."""
    e, a = math.radians(elevation_deg), math.radians(azimuth_deg)
    return (math.cos(e) * math.cos(a), math.cos(e) * math.sin(a), math.sin(e))


def yaw_quaternion(yaw):
    return (0.0, 0.0, math.sin(yaw / 2.0), math.cos(yaw / 2.0))


class StraightPass:
    """Constant-velocity pass at fixed altitude, nadir pointing."""

    def __init__(self, start, velocity, light, intensity, yaw=0.0):
        self.p0 = np.asarray(start, np.float64)
        self.v = np.asarray(velocity, np.float64)
        self.light = tuple(light)
        self.intensity = float(intensity)
        self.q = yaw_quaternion(yaw)

    def state(self, t):
        p = self.p0 + self.v * t
        return dict(position=tuple(p), velocity=tuple(self.v), light=self.light, light_rate=(0.0, 0.0, 0.0),
                    rotation=self.q, intensity=self.intensity, intensity_rate=0.0)


class Descent:
    """Linear descent from z0 to z1 over `duration` while translating along x."""

    def __init__(self, xy0, z0, z1, duration, ground_speed, light, intensity):
        self.xy0 = np.asarray(xy0, np.float64)
        self.z0, self.z1, self.T = float(z0), float(z1), float(duration)
        self.vx = float(ground_speed)
        self.light = tuple(light)
        self.intensity = float(intensity)

    def state(self, t):
        vz = (self.z1 - self.z0) / self.T
        p = (self.xy0[0] + self.vx * t, self.xy0[1], self.z0 + vz * t)
        return dict(position=p, velocity=(self.vx, 0.0, vz), light=self.light, light_rate=(0.0, 0.0, 0.0),
                    rotation=(0.0, 0.0, 0.0, 1.0), intensity=self.intensity, intensity_rate=0.0)


class Orbit:
    """Constant-altitude arc: speed v along a heading that turns at yaw_rate."""

    def __init__(self, xy0, altitude, speed, heading, yaw_rate, light, intensity):
        self.xy0 = np.asarray(xy0, np.float64)
        self.h, self.v, self.psi0, self.w = float(altitude), float(speed), float(heading), float(yaw_rate)
        self.light = tuple(light)
        self.intensity = float(intensity)

    def state(self, t):
        psi = self.psi0 + self.w * t
        if abs(self.w) > 1e-12:
            x = self.xy0[0] + self.v / self.w * (math.sin(psi) - math.sin(self.psi0))
            y = self.xy0[1] - self.v / self.w * (math.cos(psi) - math.cos(self.psi0))
        else:
            x = self.xy0[0] + self.v * t * math.cos(psi)
            y = self.xy0[1] + self.v * t * math.sin(psi)
        vel = (self.v * math.cos(psi), self.v * math.sin(psi), 0.0)
        return dict(position=(x, y, self.h), velocity=vel, light=self.light, light_rate=(0.0, 0.0, 0.0),
                    rotation=yaw_quaternion(psi), intensity=self.intensity, intensity_rate=0.0)


def horizons(trajectory, t_start, step, count, float_step=True):
    """`count` contiguous intervals [t_k, t_k+1] with t_k = t_start + k*step.

    With float_step the step is first rounded to float, as the reference app
    holds scene.time_resolution in a float (apps/main_dvs.cpp:302), so a
    1e-6 s horizon spans exactly one 1e-6 circuit cell (also a float)."""
    if float_step:
        step = float(np.float32(step))
    out = []
    prev = trajectory.state(t_start)
    t_prev = float(t_start)
    for k in range(1, count + 1):
        t = float(t_start) + k * float(step)
        cur = trajectory.state(t)
        out.append((prev, cur, t_prev, t))
        prev, t_prev = cur, t
    return out
