"""Default run options and the canned symmetry-point paths of the reference's Options
(src/EPP/Options.cpp:5-31)."""

NR_THREADS = 4
MATERIAL_NAME = "Si"
NR_POINTS = 60
NEAREST_NEIGHBORS = 12
NR_LEVELS = 30
PATH_NO = 1

DEFAULT_PATHS = [
    "KWXGLW", "WGXWLG", "WLGXWK", "LGXKG", "LGXWKG", "LGXUKG", "LGXUG", "LKWGXWLGK", "GXKGLKWX", "GXWLGKWU",
    "GXWLGK", "GXWLGKX", "GXWLGX", "GXWGUX", "GXWKLG", "GXWKGLUWLK", "GXUKGLWX",
]
