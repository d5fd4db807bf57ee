"""Exceptions of the host API, named after the reference's exception types
(src/util/Exception.h) so that callers' error handling reads the same."""


class Exception_(Exception):
    """Base of all library errors (the reference's Lab::Exception)."""


class InvalidParameterException(Exception_):
    pass


class InvalidValueException(Exception_):
    pass


class InvalidStateException(Exception_):
    pass


class MissingValueException(Exception_):
    pass


class CUDAException(Exception_):
    pass


class UnsupportedException(Exception_):
    pass


class OutOfMemoryException(CUDAException):
    pass


class DeviceTimeoutException(CUDAException):
    pass


class NativeLibraryError(Exception_):
    """libusgb.so is missing or cannot be loaded (there is no CPU fallback)."""


_BY_STATUS = {
    1: InvalidParameterException,
    2: InvalidValueException,
    3: InvalidStateException,
    4: CUDAException,
    5: UnsupportedException,
    6: OutOfMemoryException,
    7: DeviceTimeoutException,
}


def from_status(code: int, msg: str) -> Exception_:
    return _BY_STATUS.get(code, Exception_)(msg or f"usgb status {code}")
