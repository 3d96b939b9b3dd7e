"""Oracle-side exception mirroring `edelweissfe/utils/exceptions.py:44-49` (CutbackRequest)."""


class CutbackRequest(Exception):
    """Raised when a material point asks for a smaller increment (reference: utils/exceptions.py:44-49)."""

    def __init__(self, message, cutbackSize):
        super().__init__(message)
        self.cutbackSize = cutbackSize
