def get_cython_function_address(*args, **kwargs):
    raise ImportError("numba stand-in: no cython function addresses")
