"""Warning categories of the public API (reference: python/cpm/warnings.py:12-36)."""


class CPMInitializationWarning(UserWarning):
    """A run fell back to the default scatter-and-grow placement.

    The starting contact topology changes how much burn-in a run needs, so
    choosing it silently would be an unrecorded modelling decision. Silence
    it with ``warnings.simplefilter("ignore", CPMInitializationWarning)`` or
    ``CPM.initialize(warn_on_default_init=False)``.
    """


class CPMLowResolutionWarning(UserWarning):
    """``cells_for_density`` was asked for cells whose implied radius is
    under about five lattice sites, where the lattice discretisation starts
    to dominate the shape readouts."""
