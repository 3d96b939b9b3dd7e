"""Exceptions mirroring `edelweissfe/utils/exceptions.py`."""


class CutbackRequest(Exception):
    """A material point asked for a smaller increment (reference: utils/exceptions.py:44-49).

    Raised on the host when the device status word reports EFE_STATUS_CUTBACK."""

    def __init__(self, message, cutbackSize):
        super().__init__(message)
        self.cutbackSize = cutbackSize
