"""File-backed memoisation, as general results are cached by the reference (utils.py:9-25)."""

from __future__ import annotations

import logging
import pathlib
from os.path import isfile

_logger = logging.getLogger(__name__)


def load_calculate_save(*paths: pathlib.Path, load_fun, calc_fun, save_fun):
    """Load the result if every path exists, else calculate and save it (same contract as the reference)."""
    already_exist = all(isfile(path) for path in paths)
    str_paths = [str(p) for p in paths]
    if already_exist:
        try:
            result = load_fun(*paths)
            _logger.debug(f"loaded {str_paths}")
        except OSError as e:
            raise OSError(f"Loading {str_paths}: file(s) exists but load failed. {e}") from e
    else:
        _logger.debug(f"starting calculating {str_paths}")
        result = calc_fun()
        save_fun(result, *paths)
        _logger.debug(f"finished calculating {str_paths}")
    return result
