set output "hist_cfg1_MOTIF00005.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-36.9012:9.92529]
set yrange [0:123328]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00005.dat" using 1:2 title 'MOTIF00005 (cfg1)' with boxes
