"""fourierflows.jl_gb300 -- FourierFlows.jl's pseudospectral time-stepping path on GB300.

The public names mirror the Julia package (src/FourierFlows.jl:10-61).  Julia's mutating
``f!`` functions are spelled ``f_`` (PyTorch's in-place convention): ``stepforward_``,
``step_until_``, ``dealias_``, ``mul_``, ``ldiv_``, ``increment_``, ``update_``,
``extend_``; the Diffusion module has ``set_c_`` and ``updatevars_``.  Arrays use the
reference's column-major shapes (see ``devices``); all GPU compute is in
libfourierflows_gb300.so (``csrc/``, C ABI in ``include/fourierflows_gb300.h``).
"""
from . import _lib
from .devices import CPU, GPU, Device, cxtype, device_array, fltype, to_numpy, zeros
from .domains import (AbstractGrid, DomainError, OneDGrid, ThreeDGrid, TwoDGrid, dealias_, getaliasedwavenumbers,
                      gridpoints, makefilter)
from .plans import FFTPlan, RFFTPlan, fft, ifft, irfft, ldiv_, mul_, plan_flows_fft, plan_flows_rfft, rfft
from .problem import AbstractParams, AbstractVars, Clock, EmptyParams, EmptyVars, Equation, Problem, supersize
from .timesteppers import (AB3TimeStepper, AbstractTimeStepper, ETDRK4TimeStepper, FilteredAB3TimeStepper,
                           FilteredETDRK4TimeStepper, FilteredForwardEulerTimeStepper, FilteredLSRK54TimeStepper,
                           FilteredRK4TimeStepper, ForwardEulerTimeStepper, LSRK54TimeStepper, RK4TimeStepper,
                           TimeStepper, getetdcoeffs, getexpLs, isexplicit, step_until_, stepforward_)
from .utils import (innereltype, jacobian, jacobianh, on_grid, parsevalsum, parsevalsum2, radialspectrum,
                    superzeros)
from .diagnostics import AbstractDiagnostic, Diagnostic, extend_, increment_, update_
from . import diffusion as Diffusion
from . import vorticity as Vorticity
from . import adjoint as Adjoint
from .output import Output, flush, openoutput, savediagnostic, saveoutput, saveproblem, uniquepath, withoutjld2
from .adjoint import rrule_stepforward

__version__ = "0.1.0"


def native_library_path():
    return _lib.LIBPATH
