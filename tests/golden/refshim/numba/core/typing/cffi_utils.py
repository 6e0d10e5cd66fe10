def register_module(mod):
    return None
