"""Exception taxonomy of the reference, mapped from C-ABI status codes.

ShapeError and DimensionError mirror src/exceptions/exceptions.cr:4-22
(DimensionError is a ShapeError).  Crystal's stdlib IndexError, OverflowError
and DivisionByZeroError map onto Python's IndexError, OverflowError and
ZeroDivisionError; ArgumentError onto ValueError; Enumerable::EmptyError onto
EmptyError (a ValueError).
"""


class ShapeError(Exception):
    """Raised when the shape of an operand is wrong for an operation."""

    def __init__(self, message=None):
        super().__init__(message or "Shape was invalid for this operation.")


class DimensionError(ShapeError):
    """Raised when the number of dimensions is wrong for an operation."""

    def __init__(self, message=None):
        super().__init__(message or "Wrong number of dimensions for this operation.")


class ArgumentError(ValueError):
    pass


class EmptyError(ValueError):
    pass


class DivisionByZeroError(ZeroDivisionError):
    pass


class DeviceError(RuntimeError):
    """A CUDA failure or a device-side time-out."""


def from_status(code, message):
    from . import _abi as a

    table = {
        a.ERR_SHAPE: ShapeError,
        a.ERR_DIM: DimensionError,
        a.ERR_INDEX: IndexError,
        a.ERR_OVERFLOW: OverflowError,
        a.ERR_DIVZERO: DivisionByZeroError,
        a.ERR_ARGUMENT: ArgumentError,
        a.ERR_UNBOUNDED: ValueError,
        a.ERR_EMPTY: EmptyError,
        a.ERR_UNSUPPORTED: NotImplementedError,
        a.ERR_OOM: MemoryError,
    }
    return table.get(code, DeviceError)(message)
