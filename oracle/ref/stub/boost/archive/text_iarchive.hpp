#pragma once
namespace boost { namespace archive { class text_iarchive {}; }}
