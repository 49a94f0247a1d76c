"""ctypes signatures of the drop-in wrappers (include/Particle_cuda.cuh): the
package's binding, stellarsolver_gb300.dropin."""
from stellarsolver_gb300.dropin import load  # noqa: F401
