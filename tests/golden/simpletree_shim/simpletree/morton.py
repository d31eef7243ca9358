import numpy as np


def get_key_params(box, c0, L0):
    raise NotImplementedError("keys are not used by the fixture generator")
