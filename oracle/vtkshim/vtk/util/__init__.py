"""Stand-in ``vtk.util`` (see the package docstring) -- TEST INFRASTRUCTURE ONLY."""
