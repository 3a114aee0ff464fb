"""Per-solver loggers named ``rkstiff.<Class>`` (the names rkstiff/util/loghelper.py:190-219 uses)."""

from __future__ import annotations

import logging
from typing import Union

_LEVEL_NAMES = {
    logging.DEBUG: "DEBUG",
    logging.INFO: "INFO",
    logging.WARNING: "WARNING",
    logging.ERROR: "ERROR",
    logging.CRITICAL: "CRITICAL",
}


def parse_loglevel(loglevel: Union[str, int]) -> int:
    """Accept 'DEBUG'..'CRITICAL' (any case) or a logging constant; ValueError otherwise."""
    if isinstance(loglevel, str):
        level = getattr(logging, loglevel.upper(), None)
        if not isinstance(level, int):
            raise ValueError(f"Invalid log level: {loglevel}")
        return level
    return int(loglevel)


def get_level_name(level: int) -> str:
    return _LEVEL_NAMES.get(level, f"Level {level}")


def setup_logger(name: str, loglevel: Union[str, int] = "WARNING") -> logging.Logger:
    logger = logging.getLogger(name)
    logger.setLevel(parse_loglevel(loglevel))
    if not logger.handlers:
        handler = logging.StreamHandler()
        handler.setFormatter(logging.Formatter("%(asctime)s - %(name)s - %(levelname)s - %(message)s",
                                               datefmt="%Y-%m-%d %H:%M:%S"))
        logger.addHandler(handler)
    return logger


def set_log_level(logger: logging.Logger, loglevel: Union[str, int]) -> None:
    logger.setLevel(parse_loglevel(loglevel))


def get_solver_logger(solver_class: type, loglevel: Union[str, int] = "WARNING") -> logging.Logger:
    return setup_logger(f"rkstiff.{solver_class.__name__}", loglevel)
