"""placeholder"""
class PyCombustionKernels:
    def __getattr__(self, name):
        return lambda *a, **k: None
