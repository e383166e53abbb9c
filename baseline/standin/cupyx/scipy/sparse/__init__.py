from scipy.sparse import *  # noqa: F401,F403
