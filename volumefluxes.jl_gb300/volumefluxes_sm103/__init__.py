"""volumefluxes_sm103 -- VolumeFluxes.jl's 2D shallow-water step on GB300 (sm_103a).

The scenario API mirrors the reference (see api.py); the compute path is
libvfsm103.so, whose C ABI is declared in include/volumefluxes_sm103.h.
"""
from .api import (  # noqa: F401
    XDIR, YDIR, ArgumentError, DomainError,
    BoundaryCondition, PeriodicBC, WallBC, NeumannBC, CartesianGrid,
    compute_dx, compute_dy, cell_faces, cell_centers, cell_center,
    ConstantBottomTopography, BottomTopography2D, is_zero, B_cell, B_face_left, B_face_right,
    collect_topography_cells,
    ShallowWaterEquations, conserved_variable_names, desingularize,
    Reconstruction, LinearReconstruction, NoReconstruction, minmod,
    NumericalFlux, CentralUpwind,
    SourceTerm, SourceTermBottom, SourceTermRain, SourceTermInfiltration, ConstantRain, ConstantInfiltration,
    TimeDependentRain, FunctionalRain, HortonInfiltration,
    compute_rain, compute_infiltration,
    friction_bsa2012, friction_fcg2016, friction_bh2021, ImplicitFriction,
    TimeStepper, RungeKutta2, ForwardEulerStepper, number_of_substeps,
    SM103Backend, name, get_available_backends, convert_to_backend,
    System, ConservedSystem, StateView, Simulator, system_config,
    set_current_state, current_state, current_interior_state, current_time, current_timestep,
    perform_step, water_volume, simulate_to_time, IntervalWriter, MultipleCallbacks, sample_cells, GaugeRecorder,
)
from ._native import library_path, load as load_library  # noqa: F401
