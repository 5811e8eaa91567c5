"""Host-side mirror of the reference's configuration and I/O layer.

The reference keeps these parts in Fortran on the host (namelists read by
vars_module/domain_module/..., netCDF through io_module, time-chunked input
through memchunk_module, output cadence through diagTask).  They are outside
the accelerated path; this package restates just enough of them to drive the
C ABI from Python with the reference's own selfcheck configurations.
"""
