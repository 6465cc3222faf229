"""Host mirror of casa-imaging's gridder/imaging/deconvolver seams over the
GB300 CUDA library (libcasars_cuda.so).  See imaging.py for the API."""
from ._lib import CasarsCudaError, load as load_library  # noqa: F401
from .imaging import (Context, GridSums, HogbomOutcome, ImageGeometry, Plan, PsfState,  # noqa: F401
                      StandardGridder, VisibilityBatch, WProjector, adjoint, apply_weighting,
                      degrid, dirty_image, grid_dirty, grid_residual, grid_to_image,
                      image_to_grid, predict, residual_image, run_hogbom_minor_cycle,
                      CubeBatch, cube_degrid, cube_grid_degrid, cube_grid_dirty,
                      cube_sample_taps, CubePlan, BeamFit, fit_beam, restore, psf_sidelobe,
                      RowRuns, Polarization, prepare_row_runs, apply_weighting_rows,
                      run_hogbom_planes, run_clark_minor_cycle, clark_ncent,
                      DirtyAccumulator, hogbom_plane_minor_cycle, robust_rms, nsigma_threshold,
                      probe_tap_rate, Multiscale, MultiscaleOutcome, RowFeed, RowBlockSlot,
                      ReadAheadSummary, stream_row_blocks, append_hogbom_trace)
from .clean import (CleanConfig, CleanResult, clean_cycle_threshold, run_cotton_schwab,  # noqa: F401
                    CubeCleanResult, cube_clean_loop, run_cube_clean, run_clark_cotton_schwab,
                    run_multiscale_cotton_schwab,
                    HogbomPlaneMinorCycleControl, HogbomPlaneComponent,
                    HogbomPlaneMinorCycleOutcome, run_hogbom_plane_minor_cycle)
from .run import (ImagingRequest, ImagingResult, StandardMfsDirtyGridResult,  # noqa: F401
                  finish_standard_mfs_dirty_grid_result, run_imaging,
                  run_standard_mfs_dirty_grid_plan, run_standard_mfs_plan)
