"""3-vector helpers the reference's nmag namespace carries
(interface/nsim/vectools.py)."""
import math

__all__ = ["normalised_vector", "vector3_dot", "vector3_cross"]


def vector3_dot(v, w):
    return v[0] * w[0] + v[1] * w[1] + v[2] * w[2]


def vector3_cross(v, w):
    return (v[1] * w[2] - v[2] * w[1], v[2] * w[0] - v[0] * w[2], v[0] * w[1] - v[1] * w[0])


def normalised_vector(vector):
    """The vector divided by its length (a list)."""
    inv = 1.0 / math.sqrt(vector3_dot(vector, vector))
    return [x * inv for x in vector]
