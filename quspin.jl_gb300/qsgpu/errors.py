"""Exceptions mirroring the Julia exceptions the reference raises on this path."""


class ArgumentError(ValueError):
    """Julia ArgumentError."""


class DimensionMismatch(ValueError):
    """Julia DimensionMismatch."""


class ErrorException(RuntimeError):
    """Julia ErrorException (non-convergence, device failure)."""


class UnsupportedError(ArgumentError):
    """A request outside what this engine implements (raised as ArgumentError)."""


def raise_status(status: int, message: str):
    if status == 1:
        raise ArgumentError(message)
    if status == 2:
        raise DimensionMismatch(message)
    if status == 4:
        raise MemoryError(message)
    if status == 6:
        raise UnsupportedError(message)
    if status in (3, 5, 7):
        raise ErrorException(message)
    raise ErrorException(f"status {status}: {message}")
