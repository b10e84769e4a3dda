"""ctypes mirror of include/eulersf.h (structs, enums, field table)."""
from __future__ import annotations

import ctypes as C

import numpy as np

ESF_MAX_SOLIDS = 8

STATUS = {
    0: "ESF_OK", 1: "ESF_ERR_INVALID_ARG", 2: "ESF_ERR_STATE", 3: "ESF_ERR_CUDA",
    4: "ESF_ERR_OOM", 5: "ESF_ERR_IO", 6: "ESF_ERR_NUMERIC", 7: "ESF_ERR_NO_DEVICE",
    8: "ESF_ERR_UNSUPPORTED",
}
ESF_FP64, ESF_MIXED, ESF_MIXED_X64 = 0, 1, 2


class EsfError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)} {detail}".strip())


class Grid(C.Structure):
    _fields_ = [("xRes", C.c_int), ("yRes", C.c_int), ("zRes", C.c_int),
                ("dh", C.c_double), ("origin", C.c_double * 3)]


class Params(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("fluid_density", C.c_double), ("fluid_viscosity", C.c_double),
        ("vorticity_eps", C.c_double), ("buoyancy", C.c_double), ("gravity", C.c_double),
        ("rayleigh_alpha", C.c_double), ("rayleigh_beta", C.c_double),
        ("implicit_solver_eps", C.c_double), ("div_free_solver_eps", C.c_double),
        ("cr_max_iterations", C.c_int), ("mass_sample_dh", C.c_double),
        ("tight_border", C.c_int), ("extrapolation_cells", C.c_int),
        ("particles_per_cell", C.c_int), ("flip_alpha", C.c_double),
        ("contact_safe_distance", C.c_double), ("wall_thickness", C.c_double),
        ("contact_spring_stiffness", C.c_double), ("friction", C.c_double),
        ("flip_cutoff", C.c_int), ("flow_rate", C.c_double),
        ("precision", C.c_int), ("inner_eps", C.c_double), ("max_refinements", C.c_int),
    ]


class SolidDesc(C.Structure):
    _fields_ = [
        ("mass_res", C.c_int * 3), ("mass_dh", C.c_double), ("mass_origin", C.c_double * 3),
        ("rest_mass", C.POINTER(C.c_double)), ("lambda_", C.c_double), ("mu", C.c_double),
        ("density", C.c_double), ("rotation", C.c_double * 9), ("translation", C.c_double * 3),
        ("scaling", C.c_double * 3), ("initial_velocity", C.c_double * 3),
        ("num_vertices", C.c_int), ("vertices", C.POINTER(C.c_double)),
        ("num_triangles", C.c_int), ("triangles", C.POINTER(C.c_int)),
        ("plastic_yield", C.c_double),
    ]


class StepReport(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("energy", C.c_double), ("iterations", C.c_int * 3),
        ("converged", C.c_int * 3), ("rel_residual", C.c_double * 3),
        ("refinements", C.c_int * 3), ("fp64_iterations", C.c_int), ("prone_to_contact", C.c_int),
        ("num_particles", C.c_int), ("status", C.c_int), ("device_ms", C.c_double),
        ("phase_ms", C.c_double * 13), ("fp64_stress_cells", C.c_int), ("valid_cells", C.c_int),
        ("solid_contacts", C.c_int),
    ]
    PHASES = ["broad_phase_cfl", "solid_forces_stiffness", "body_forces", "solid_solve_1",
              "pressure_solve", "solid_solve_2", "grid_to_particle", "particle_to_grid",
              "velocity_extension", "solid_displacement", "solid_mass", "mesh_sdf_particles",
              "fluid_advection"]

    def as_dict(self) -> dict:
        return {
            "dt": self.dt, "energy": self.energy, "iterations": list(self.iterations),
            "converged": list(self.converged), "rel_residual": list(self.rel_residual),
            "refinements": list(self.refinements), "fp64_iterations": self.fp64_iterations,
            "prone_to_contact": self.prone_to_contact,
            "num_particles": self.num_particles, "status": self.status,
            "device_ms": self.device_ms, "fp64_stress_cells": self.fp64_stress_cells,
            "valid_cells": self.valid_cells,
            "solid_contacts": self.solid_contacts,
            "phase_ms": dict(zip(self.PHASES, list(self.phase_ms))),
        }


# field id -> (name, numpy dtype, components per entry for reshaping)
FIELDS = {
    "velocity": (0, np.float64, 3), "intensity": (1, np.float64, 1),
    "solidMass": (2, np.float64, 1), "nodeSolidVolumeFraction": (3, np.float64, 1),
    "gridIdxToSolutionIdx": (4, np.int32, 1), "gridIdxToSolidIdx": (5, np.int32, 1),
    "lambda1": (10, np.float64, 1), "JMInvJTDiag": (11, np.float64, 1),
    "divergenceConstraintsRHS": (12, np.float64, 1), "b1": (13, np.float64, 1),
    "nzMassVecInv": (20, np.float64, 1), "velocityAtDt0": (21, np.float64, 1),
    "velocityAtDt1": (22, np.float64, 1), "unitForce": (23, np.float64, 1),
    "solidUnitForce": (30, np.float64, 1), "solidVelocityAtDt0": (31, np.float64, 1),
    "solidPressureCorrection": (32, np.float64, 1), "dampedSolidMassVec": (33, np.float64, 1),
    "systemDiag": (34, np.float64, 1), "systemBlocks": (35, np.float64, 1),
    "systemMask": (36, np.int32, 1),
    "solid.u": (50, np.float64, 3), "solid.X": (51, np.float64, 3),
    "solid.velocity": (52, np.float64, 3), "solid.vecWorkspace": (53, np.float64, 3),
    "solid.mass": (54, np.float64, 1), "solid.phi": (55, np.float64, 1),
    "solid.detFInv": (56, np.float64, 1), "solid.valid": (57, np.int8, 1),
    "solid.quarterVolumeFractions": (58, np.float64, 1),
    "solid.particles": (59, np.float64, 10), "solid.meshVertices": (60, np.float64, 3),
    "solid.boxes": (61, np.int32, 1),
    "solid.FpInv": (62, np.float64, 9), "solid.FpInvGrid": (63, np.float64, 1),
}


def declare(lib: C.CDLL, prefix: str, device_pointer_ops: bool) -> None:
    """Set argtypes/restype of the scene API exported with `prefix`."""
    vp = C.c_void_p
    f = lambda n: getattr(lib, prefix + n)
    f("create").restype = vp
    f("destroy").argtypes = [vp]
    f("add_solid").argtypes = [vp, C.POINTER(SolidDesc)]
    f("set_fluid").argtypes = [vp, C.c_double, C.c_double]
    f("init").argtypes = [vp]
    f("set_max_dt").argtypes = [vp, C.c_double]
    f("step").argtypes = [vp, C.POINTER(StepReport)]
    f("dt").argtypes = [vp]
    f("dt").restype = C.c_double
    f("field_info").argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_size_t),
                                C.POINTER(C.c_size_t)]
    f("get_field").argtypes = [vp, C.c_int, C.c_int, vp, C.c_size_t]
    f("set_field").argtypes = [vp, C.c_int, C.c_int, vp, C.c_size_t]
    f("params_default").argtypes = [C.POINTER(Grid), C.POINTER(Params)]
