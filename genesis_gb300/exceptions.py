"""Exception type of the package (the reference raises genesis.GenesisException)."""


class GenesisException(Exception):
    pass


class DeprecationError(GenesisException):
    """A removed option or property (genesis/utils/misc.py DeprecationError)."""
