"""Warning categories of the public interface (odtbrain/warn.py): the
reference defines them for callers to filter on; nothing here raises
them."""


class DataUndersampledWarning(UserWarning):
    """Sinogram data undersampled for the requested reconstruction."""


class ImplementationAmbiguousWarning(UserWarning):
    """A parameter combination the reference implements ambiguously."""
