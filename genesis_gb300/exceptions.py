"""Exception type of the package (the reference raises genesis.GenesisException)."""


class GenesisException(Exception):
    pass
