"""INI configuration with evaluated values, as pyprop reads it.

Restates pyprop/Config.py:4-117:
  * every option value is a Python expression evaluated in the project
    namespace (the __main__ module plus this package's globals), with the
    section's already-parsed options as locals (Config.py:19-29);
  * `base = "Other"` pulls in another section's options first (Config.py:11-17);
  * `[Import] files = [...]` recursively loads other INI files, imported files
    first (Config.py:85-117);
  * `%(key)s` interpolation from the same section (ConfigParser).
"""
from __future__ import annotations

import configparser
import os
import sys


def _project_namespace():
    ns = {}
    # package names first, then __main__ (the user's project wins)
    from . import namespace as _pkgns
    ns.update(_pkgns.eval_namespace())
    main = sys.modules.get("__main__")
    if main is not None:
        ns.update(getattr(main, "__dict__", {}))
    return ns


class Section:
    def __init__(self, name, cfg=None):
        self.name = name
        if cfg is not None:
            self.LoadConfig(name, cfg)

    def LoadConfig(self, name, cfg):
        for optionName in cfg.options(name):
            if optionName == "base":
                importName = eval(cfg.get(name, optionName))
                self.LoadConfig(importName, cfg)
            else:
                self.SetOptionString(optionName, cfg.get(name, optionName))

    def SetOptionString(self, optionName, optionString):
        glob = _project_namespace()
        optionValue = eval(optionString, glob, self.__dict__)
        self.Set(optionName, optionValue)

    def Set(self, optionName, optionValue):
        if optionName in ["name", "SetOptionString", "Set", "Get"]:
            raise Exception("Invalid optionName %s" % optionName)
        self.__dict__[optionName] = optionValue

    def Get(self, optionName):
        return self.__dict__[optionName]

    def get(self, optionName, default=None):
        return self.__dict__.get(optionName, default)

    def Exists(self, optionName):
        return hasattr(self, optionName)

    def __getitem__(self, key):
        return self.__dict__[key]

    def Apply(self, other):
        if hasattr(other, "ApplyConfigSection"):
            other.ApplyConfigSection(self)


class Config:
    def __init__(self, cfg):
        self.cfgObj = cfg
        for sectionName in cfg.sections():
            if sectionName in ["GetSection"]:
                raise Exception("Invalid sectionName %s" % sectionName)
            section = Section(sectionName, cfg)
            section.Config = self
            self.__dict__[sectionName] = section

    def GetSection(self, sectionName):
        return self.__dict__[sectionName]

    def Apply(self, other):
        if hasattr(other, "ApplyConfig"):
            other.ApplyConfig(self)

    def SetValue(self, section, optionName, value, infoLevel=0, ignoreSerializationError=False):
        try:
            eval(repr(value), _project_namespace())
        except Exception:
            if not ignoreSerializationError:
                raise Exception("Object cannot be serialized: %s" % repr(value))
        self.cfgObj.set(section, optionName, repr(value))
        self.__dict__[section].Set(optionName, value)
        if infoLevel > 0:
            print("Changing %s.%s to %s" % (section, optionName, value))


def _parser():
    return configparser.ConfigParser(interpolation=configparser.BasicInterpolation())


def Load(fileName, silent=True):
    """pyprop.Load (Config.py:85-117)."""
    configFiles = []
    newFiles = [(".", fileName)]
    while newFiles:
        curDir, curFile = newFiles.pop()
        localFile = curDir.rstrip("/") + "/" + curFile if not os.path.isabs(curFile) else curFile
        absFile = os.path.abspath(os.path.expanduser(os.path.expandvars(localFile)))
        absDir = os.path.dirname(absFile)
        if not silent:
            print("Using config file", absFile)
        configFiles.insert(0, absFile)
        cfg = _parser()
        with open(absFile) as f:
            cfg.read_file(f)
        if cfg.has_section("Import") and cfg.has_option("Import", "files"):
            for f in eval(cfg.get("Import", "files")):
                newFiles.insert(0, (absDir, f))
    cfg = _parser()
    for file in configFiles:
        with open(file) as f:
            cfg.read_file(f)
    return Config(cfg)


def LoadString(text):
    """Parse a configuration given as a string (same semantics as Load, no [Import])."""
    cfg = _parser()
    cfg.read_string(text)
    return Config(cfg)
