set output "hist_cfg1_MOTIF00004.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-44.7223:13.56]
set yrange [0:2061]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00004.dat" using 1:2 title 'MOTIF00004 (cfg1)' with boxes
