"""Imfit configuration files (the format of core/config_file_parser.cpp:494-657).

Lines are trimmed; empty lines and lines starting with '#' are skipped, and
'#' starts a comment anywhere.  Lines before the first ``X0`` are image
options ``NAME value`` (GAIN, READNOISE, ORIGINAL_SKY, EXPTIME, NCOMBINED).
The function section is a sequence of function sets, each opened by
``X0 value [limits]`` and ``Y0 value [limits]``, followed by ``FUNCTION name``
blocks whose parameter lines are ``name value [lo,hi | fixed]``.  A
``# LABEL text`` comment on a FUNCTION line labels that function
(core/config_file_parser.cpp:208-222), and an ``OPTIONAL_PARAMS_START`` ...
``OPTIONAL_PARAMS_END`` block after it holds ``name value`` pairs for the
function's optional parameters (core/config_file_parser.cpp:450-465).
"""
from dataclasses import dataclass, field

import numpy as np

_OPTION_NAMES = {"GAIN", "READNOISE", "ORIGINAL_SKY", "EXPTIME", "NCOMBINED"}


@dataclass
class ModelConfig:
    options: dict = field(default_factory=dict)
    functions: list = field(default_factory=list)   # [(name, starts_new_set)]
    labels: list = field(default_factory=list)      # per function, "" when unlabelled
    optional: list = field(default_factory=list)    # per function, {name: value}
    param_names: list = field(default_factory=list)
    values: np.ndarray = None
    lower: np.ndarray = None                          # NaN: no limit
    upper: np.ndarray = None
    fixed: np.ndarray = None                          # 1 = fixed

    @property
    def gain(self):
        return float(self.options.get("GAIN", 1.0))

    @property
    def read_noise(self):
        return float(self.options.get("READNOISE", 0.0))

    @property
    def original_sky(self):
        return float(self.options.get("ORIGINAL_SKY", 0.0))

    @property
    def exp_time(self):
        return float(self.options.get("EXPTIME", 1.0))

    @property
    def n_combined(self):
        return int(float(self.options.get("NCOMBINED", 1)))


class ConfigError(ValueError):
    pass


def _strip(line):
    return line.split("#", 1)[0].strip()


def _label(line):
    k = line.find("LABEL")
    return "" if k < 0 else line[k + 5:].strip()


def parse_config(text, check_limits=True):
    """Parse the text of an Imfit configuration file.  check_limits=False is
    makeimage's reading (ReadConfigFile in makeimage mode): limits are kept
    but not checked against the values."""
    lines = []
    for k, raw in enumerate(text.splitlines(), 1):
        t = raw.strip()
        if t and not t.startswith("#"):
            lines.append((k, _strip(t), t))
    cfg = ModelConfig()
    i = 0
    while i < len(lines) and lines[i][1].split()[0] != "X0":
        parts = lines[i][1].split()
        if parts[0] == "FUNCTION":
            raise ConfigError(f"line {lines[i][0]}: FUNCTION before the first X0")
        if len(parts) == 2:
            cfg.options[parts[0]] = parts[1]
        i += 1
    if i == len(lines):
        raise ConfigError("no function section (X0 line) found")
    vals, lo, hi, fx = [], [], [], []
    new_set = False
    expecting_y0 = False

    def param(lineno, parts):
        if len(parts) < 2:
            raise ConfigError(f"line {lineno}: parameter line needs a value")
        try:
            v = float(parts[1])
        except ValueError:
            raise ConfigError(f"line {lineno}: bad parameter value {parts[1]!r}")
        lim = parts[2] if len(parts) > 2 else None
        l, h, f = np.nan, np.nan, 0
        if lim is not None:
            if lim.lower() == "fixed":
                f = 1
            else:
                try:
                    a, b = (float(x) for x in lim.split(","))
                except ValueError:
                    raise ConfigError(f"line {lineno}: bad limits {lim!r}")
                if check_limits and a >= b:  # equal limits are an error too: "fixed" holds a value
                    raise ConfigError(f"line {lineno}: first parameter limit ({a:g}) must be < second limit "
                                      f"({b:g})")
                if check_limits and not (a <= v <= b):
                    raise ConfigError(f"line {lineno}: initial value outside its limits")
                l, h = a, b
        cfg.param_names.append(parts[0])
        vals.append(v)
        lo.append(l)
        hi.append(h)
        fx.append(f)

    in_optional = False
    for lineno, text_, raw in lines[i:]:
        parts = text_.split()
        key = parts[0]
        if key == "OPTIONAL_PARAMS_START":
            if not cfg.functions or in_optional:
                raise ConfigError(f"line {lineno}: OPTIONAL_PARAMS_START outside a function")
            in_optional = True
        elif key == "OPTIONAL_PARAMS_END":
            if not in_optional:
                raise ConfigError(f"line {lineno}: OPTIONAL_PARAMS_END without a start")
            in_optional = False
        elif in_optional:
            if len(parts) < 2:
                raise ConfigError(f"line {lineno}: optional parameter needs a value")
            cfg.optional[-1][parts[0]] = parts[1]
        elif key == "X0":
            param(lineno, parts)
            new_set = True
            expecting_y0 = True
        elif key == "Y0":
            if not expecting_y0:
                raise ConfigError(f"line {lineno}: Y0 without X0")
            param(lineno, parts)
            expecting_y0 = False
        elif key == "FUNCTION":
            if expecting_y0:
                raise ConfigError(f"line {lineno}: X0 without Y0")
            if len(parts) < 2:
                raise ConfigError(f"line {lineno}: FUNCTION without a name")
            cfg.functions.append((parts[1], new_set))
            cfg.labels.append(_label(raw))
            cfg.optional.append({})
            new_set = False
        elif key in _OPTION_NAMES:
            raise ConfigError(f"line {lineno}: image option inside the function section")
        else:
            if not cfg.functions:
                raise ConfigError(f"line {lineno}: parameter before any FUNCTION")
            param(lineno, parts)
    if in_optional:
        raise ConfigError("OPTIONAL_PARAMS_START without an end")
    cfg.values = np.array(vals)
    cfg.lower = np.array(lo)
    cfg.upper = np.array(hi)
    cfg.fixed = np.array(fx, dtype=int)
    return cfg


def read_config(path, check_limits=True):
    with open(path) as f:
        return parse_config(f.read(), check_limits)


_NPARAMS = {"Sersic": 5, "Exponential": 4, "FlatSky": 1, "GaussianRing": 5, "Moffat": 5, "Gaussian": 4,
            "ExponentialDisk3D": 6, "FerrersBar3D": 8, "PointSource": 1, "PointSourceRot": 2,
            "TiltedSkyPlane": 3}


def format_params(cfg, params, chi2=None):
    """The best-fit parameters in configuration-file form (what imfit saves)."""
    out = []
    if chi2 is not None:
        out.append(f"# fit statistic = {chi2:.6f}")
    for k, v in cfg.options.items():
        out.append(f"{k}\t{v}")
    j = 0
    for k, (name, new_set) in enumerate(cfg.functions):
        if new_set:
            out.append("")
            for _ in range(2):
                out.append(f"{cfg.param_names[j]}\t{params[j]:.6f}")
                j += 1
        label = cfg.labels[k] if k < len(cfg.labels) else ""
        out.append(f"FUNCTION {name}" + (f"   # LABEL {label}" if label else ""))
        for _ in range(_NPARAMS[name]):
            out.append(f"{cfg.param_names[j]}\t{params[j]:.6f}")
            j += 1
    return "\n".join(out) + "\n"
